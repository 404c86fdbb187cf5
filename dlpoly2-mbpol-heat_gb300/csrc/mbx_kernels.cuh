// Internal declarations shared by the MB-pol CUDA translation units.
#pragma once

#include "mbx_common.cuh"

namespace mbx {

// Accumulator slots of the per-evaluation scalar buffer (double, device).
enum Slot {
    S_E2 = 0,       // 2B energy (internal units)
    S_E3 = 1,       // 3B energy
    S_VIR = 2,      // virial sum w.g (internal units)
    S_STRESS = 3,   // 9 stress components (3..11)
    S_JPOT = 12,    // 3 heat-current jpot components (12..14)
    S_JKIN = 15,    // 3 heat-current jkin components (15..17)
    S_NSLOTS = 18
};

// Device inputs/outputs of one MB-pol evaluation.
struct MbpolArgs {
    int nw;
    Cell cell;
    const int* list;                 // listttm2, 1-based, 3*nw
    const double *x, *y, *z;         // raw positions (heat current uses these)
    const double *vx, *vy, *vz;      // velocities or null
    const double* mono;              // imaged monomers, 9 per water
    double *fx, *fy, *fz;            // forces, accumulated
    double* ae;                      // per-atom energy, accumulated (may be null)
    double* acc;                     // S_NSLOTS scalars, accumulated
};

// Mixed-precision pass: FP32 kernels hand ill-conditioned clusters (a shifted
// variable further than limit2/limit3 from its centre) to an FP64 kernel through
// these device lists; count[0] dimers, count[1] trimers (zeroed by the caller).
struct MixedPass {
    int2* hard2;
    int4* hard3;
    int* count;
    float limit2, limit3;
};

// Fused cluster kernels (mbx_mbpol.cu).  precision: 0 FP64, 1 mixed.
cudaError_t launch_2b(const MbpolArgs& a, const int2* pairs, int npairs, int precision, const MixedPass& mp,
                      cudaStream_t s);
cudaError_t launch_3b(const MbpolArgs& a, const int4* trip, int ntrip, int precision, const MixedPass& mp,
                      cudaStream_t s);
// Isolated polynomial + model evaluation for explicit clusters (the per-call ABI).
cudaError_t launch_2b_direct(int n, const double* w1, const double* w2, double* E, double* g1, double* g2,
                             int precision, cudaStream_t s);
cudaError_t launch_3b_direct(int n, const double* w1, const double* w2, const double* w3, double* E,
                             double* g1, double* g2, double* g3, int precision, cudaStream_t s);
// jkin = sum_i (K_i + U_i) v_i over the water atoms (SOURCE/heatcurrent.f90:713-716).
cudaError_t launch_jkin(int nwat_atoms, const double* vx, const double* vy, const double* vz,
                        const double* mass, const double* ae, double* acc, cudaStream_t s);

// 1-body PS PES over H-O-H angles (mbx_pes.cu); acc14 = {E, virial, stress[9], jpot[3]}.
cudaError_t launch_ps_pes(int nang, const int* listang, const Cell& cl, const double* x, const double* y,
                          const double* z, double* fx, double* fy, double* fz, double* ae, const double* vx,
                          const double* vy, const double* vz, double* acc14, cudaStream_t s);

// M sites written into x/y/z at index listttm2[3nw-1] + i (0-based) and DMS charges
// into chge (H1, H2, M) and dp[6*nw] (mbx_pes.cu); chge/dp may be null.
cudaError_t launch_msites_dms(int nw, const int* list, const Cell& cl, double* x, double* y, double* z, double gamma,
                              double* chge, double* dp, cudaStream_t s);

__global__ void k_list_totals(int nw, const int* n2, const int* off2, const int* tcnt, const int* toff,
                              const int* flag, int* totals);

// Cell-list builder of the dimer and trimer lists (mbx_lists.cu).
struct ListBuilder {
    int cap2 = 64;      // dimer partners j > i per water
    int cap3 = 48;      // 3B neighbours per water
    int cap2_alloc = 0, cap3_alloc = 0;
    int nw_cap = 0, ncell_cap = 0;
    unsigned *key = nullptr, *skey = nullptr;
    int *idx = nullptr, *sidx = nullptr, *cstart = nullptr, *cend = nullptr;
    int *n2 = nullptr, *l2 = nullptr, *off2 = nullptr, *n3 = nullptr, *l3 = nullptr;
    int *tcnt = nullptr, *toff = nullptr, *flag = nullptr;
    void *scan_tmp = nullptr, *sort_tmp = nullptr;
    size_t scan_bytes = 0, sort_bytes = 0;
    int3 nc_last = {1, 1, 1};
    int all_pairs_last = 1;
    long launches_last = 0;  // kernels launched by the last phase1 + phase2 (CUB included)
    // external = true: the buffers above were set by the caller (fixed capacities, no
    // allocation, no cell sort: candidates are all waters); reserve() only checks sizes
    bool external = false;

    ~ListBuilder();
    void release();
    cudaError_t reserve(int nw, int ncell);
    // totals_dev[0] = #pairs, [1] = #trimers, [2] = overflow flag
    cudaError_t phase1(int nw, const int* list, const double* x, const double* y, const double* z, const Cell& cl,
                       double* mono, int* totals_dev, cudaStream_t s);
    cudaError_t phase2(int nw, const Cell& cl, const double* mono, int2* pairs, int4* trip, cudaStream_t s);
};

}  // namespace mbx
