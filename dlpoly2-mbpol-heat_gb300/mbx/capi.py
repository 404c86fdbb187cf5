"""ctypes binding of libmbx.so (include/mbx.h) -- the host-side mirror of the
reference's mbpol_forces interface.

There is no CPU fallback: if the library is missing, or no sm_103 GPU is present,
every call raises.
"""
import ctypes as C
import os
import re

import numpy as np

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REPO = os.path.dirname(PKG)
LIB_PATH = os.path.join(PKG, "_build", "libmbx.so")
HEADER = os.path.join(REPO, "include", "mbx.h")

FP64 = 0
MIXED = 1
ERR_ARG = 1
ERR_CONVERGE = 5
NSCALARS = 18
NBOXSCALARS = NSCALARS + 14
NWATERSCALARS = NSCALARS + 28
NSTEPSCALARS = NWATERSCALARS + 22
S_ENG2, S_ENG3, S_VIR, S_STRESS, S_JPOT, S_JKIN = 0, 1, 2, 3, 12, 15

_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)
_L = C.POINTER(C.c_long)
_lib = None


class MbxError(RuntimeError):
    pass


# mbx_ipi_force_fn: (user, replica, natoms, cell[9], xyz[3n], energy*, forces[3n], stress[9], moldip[n])
IPI_FORCE_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double),
                           C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double),
                           C.POINTER(C.c_double))


def polar_params_for_cell(cell):
    """mbx_polar_params_for_cell: the server's Ewald and dipole settings for a cell"""
    prm = np.zeros(15)
    load().mbx_polar_params_for_cell(_p(_f64(cell)), _p(prm))
    return prm


def ipi_run_callback(address, fn, max_steps=0):
    """mbx_ipi_run_callback with a Python force function
    fn(replica, cell[9], xyz[n, 3]) -> (energy, forces[n, 3], stress[9], moldip[n/3, 3]) in DL_POLY
    units; returns (status, steps, error text)."""
    lib = load()

    def cb(user, replica, nat, cell, xyz, energy, forces, stress, moldip):
        try:
            c = np.ctypeslib.as_array(cell, (9,)).copy()
            x = np.ctypeslib.as_array(xyz, (3 * nat,)).reshape(nat, 3).copy()
            e, f, st, md = fn(replica, c, x)
            energy[0] = float(e)
            np.ctypeslib.as_array(forces, (3 * nat,))[:] = np.asarray(f, np.float64).ravel()
            np.ctypeslib.as_array(stress, (9,))[:] = np.asarray(st, np.float64).ravel()
            np.ctypeslib.as_array(moldip, (3 * (nat // 3),))[:] = np.asarray(md, np.float64).ravel()
            return 0
        except Exception:   # reported to the caller as a failed evaluation
            return ERR_ARG

    cfn = IPI_FORCE_FN(cb)
    steps = C.c_long(0)
    err = C.create_string_buffer(256)
    rc = lib.mbx_ipi_run_callback(address.encode(), cfn, None, int(max_steps), C.byref(steps), err, 256)
    return rc, int(steps.value), err.value.decode()


def header_functions():
    """Names of every function declared in include/mbx.h."""
    with open(HEADER) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return re.findall(r"^\s*(?:int|long|void|const char\*)\s+\**\s*(\w+)\s*\(", text, flags=re.M)


def load(path=None):
    """Load libmbx.so and declare its prototypes (no GPU needed)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise MbxError("libmbx.so not built (%s); run __graft_entry__.build()" % path)
    L = C.CDLL(path)
    L.mbx_create.argtypes = [C.POINTER(C.c_void_p), C.c_int]
    L.mbx_destroy.argtypes = [C.c_void_p]
    L.mbx_destroy.restype = None
    L.mbx_error.argtypes = [C.c_void_p]
    L.mbx_error.restype = C.c_char_p
    L.mbx_set_stream.argtypes = [C.c_void_p, C.c_void_p]
    L.mbx_mbpol_forces.argtypes = [C.c_void_p, C.c_int, C.c_int, _D, C.c_int, _I, C.c_int, _D, _D, _D, _D, _D, _D,
                                   _D, _D, _D, _D, _D, _D, _D, _D, _D]
    L.mbx_mbpol_forces_device.argtypes = [C.c_void_p, C.c_int, C.c_int, _D, C.c_int, C.c_void_p, C.c_int,
                                          C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, _D]
    L.mbx_set_profiling.argtypes = [C.c_void_p, C.c_int]
    L.mbx_last_timings.argtypes = [C.c_void_p, _D, _L]
    L.mbx_set_mixed_limits.argtypes = [C.c_void_p, C.c_double, C.c_double]
    L.mbx_mbpol_forces_noalloc.argtypes = [C.c_int, C.c_int, _D, C.c_int, C.c_void_p, C.c_int] + \
        [C.c_void_p] * 11 + [_D, C.c_void_p]
    L.mbx_ps_pes_forces.argtypes = [C.c_void_p, C.c_int, _D, C.c_int, _I, C.c_int] + [_D] * 14
    L.mbx_ps_pes_forces_device.argtypes = [C.c_void_p, C.c_int, _D, C.c_int, C.c_void_p, C.c_int] + \
        [C.c_void_p] * 10 + [_D]
    L.mbx_msites_dms.argtypes = [C.c_void_p, C.c_int, _D, C.c_int, _I, C.c_int, C.c_double] + [_D] * 5
    L.mbx_msites_dms_device.argtypes = [C.c_void_p, C.c_int, _D, C.c_int, C.c_void_p, C.c_int, C.c_double] + \
        [C.c_void_p] * 5
    L.mbx_server_create.argtypes = [C.POINTER(C.c_void_p), C.c_int, C.c_int, C.c_double]
    L.mbx_server_set_spme.argtypes = [C.c_void_p, C.c_int, C.c_double]
    L.mbx_server_destroy.argtypes = [C.c_void_p]
    L.mbx_server_destroy.restype = None
    L.mbx_server_submit.argtypes = [C.c_void_p, C.c_int, C.c_int, _D, C.c_int, C.c_int] + [_D] * 7
    L.mbx_server_submit.restype = C.c_long
    L.mbx_server_wait.argtypes = [C.c_void_p, C.c_long] + [_D] * 6
    L.mbx_server_submit_step.argtypes = [C.c_void_p, C.c_int, C.c_long, C.c_int, _D, C.c_int] + [_D] * 7
    L.mbx_server_submit_step.restype = C.c_long
    L.mbx_server_wait_step.argtypes = [C.c_void_p, C.c_long] + [_D] * 7
    L.mbx_server_error.argtypes = [C.c_void_p]
    L.mbx_server_error.restype = C.c_char_p
    L.mbx_mbpol_multi.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, _I, _D] + [_D] * 12
    L.mbx_mbpol_multi_device.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, _I, _D] + [C.c_void_p] * 11 + [_D]
    L.mbx_water_forces.argtypes = [C.c_void_p, C.c_int, C.c_int, _D, C.c_int, _I, C.c_int, _I, _I, _I, C.c_int] + \
        [_D] * 12
    L.mbx_disp_setup.argtypes = [C.c_void_p, C.c_int, _D, C.c_double, C.c_double, C.c_int]
    L.mbx_disp_forces.argtypes = [C.c_void_p, C.c_int, _D, C.c_int, _I, _I] + [_D] * 14
    L.mbx_disp_forces_device.argtypes = [C.c_void_p, C.c_int, _D, C.c_int] + [C.c_void_p] * 12 + [_D]
    L.mbx_disp_lrc.argtypes = [C.c_int, _D, _I, C.c_double, C.c_double, _D, _D]
    L.mbx_polar_forces.argtypes = [C.c_void_p, C.c_int, _D, C.c_int, _D, C.c_int] + [_D] * 20
    L.mbx_polar_forces_device.argtypes = [C.c_void_p, C.c_int, _D, C.c_int, _D, C.c_int] + [C.c_void_p] * 14 + \
        [_D] + [C.c_void_p] * 4 + [_D, _D]
    L.mbx_polar_iterations.argtypes = [C.c_void_p]
    L.mbx_polar_inner_sweeps.argtypes = [C.c_void_p]
    L.mbx_polar_inner_sweeps.restype = C.c_long
    L.mbx_trim.argtypes = [C.c_void_p, C.c_double]
    L.mbx_trim.restype = C.c_double
    L.mbx_polar_timings.argtypes = [C.c_void_p, C.POINTER(C.c_float), _L]
    L.mbx_msite_redistribute.argtypes = [C.c_int, C.c_double, _D, _D, _D]
    L.mbx_water_step.argtypes = [C.c_void_p, C.c_int, C.c_int, _D, C.c_int, C.c_int, _D, _D, _D, _I, _I] + [_D] * 16
    L.mbx_set_lanes.argtypes = [C.c_void_p, C.c_int]
    L.mbx_set_precond_sweeps.argtypes = [C.c_void_p, C.c_int]
    L.mbx_set_precond_block.argtypes = [C.c_void_p, C.c_int]
    L.mbx_set_aspc.argtypes = [C.c_void_p, C.c_int, C.c_int]
    L.mbx_aspc_step.argtypes = [C.c_void_p]
    L.mbx_aspc_restart.argtypes = [C.c_void_p]
    L.mbx_set_dipole_guess.argtypes = [C.c_void_p, C.c_int]
    L.mbx_polar_field_timing.argtypes = [C.c_void_p, _D, _D, C.POINTER(C.c_long)]
    L.mbx_set_spme.argtypes = [C.c_void_p, C.c_int, C.c_double, _I]
    L.mbx_set_polar_skin.argtypes = [C.c_void_p, C.c_double]
    L.mbx_polar_list_builds.argtypes = [C.c_void_p]
    L.mbx_polar_list_builds.restype = C.c_long
    L.mbx_polar_last_pairs.argtypes = [C.c_void_p, _I, C.c_long, _L]
    L.mbx_spme_last_grid.argtypes = [C.c_void_p, _I]
    L.mbx_spme_grid_for_cell.argtypes = [_D, C.c_double, _I]
    L.mbx_spme_kspace.argtypes = [C.c_void_p, _D, C.c_int, _I, C.c_int, _D, C.c_int] + [_D] * 10
    L.mbx_fft3d.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _D]
    L.mbx_polar_params_for_cell.argtypes = [_D, _D]
    L.mbx_polar_params_for_cell.restype = None
    L.mbx_ipi_run_callback.argtypes = [C.c_char_p, IPI_FORCE_FN, C.c_void_p, C.c_long, C.POINTER(C.c_long),
                                       C.c_char_p, C.c_int]
    L.mbx_ipi_run.argtypes = [C.c_void_p, C.c_char_p, C.c_int, _D, C.c_int, C.c_long, C.POINTER(C.c_long)]
    L.mbx_water_step_multi.argtypes = ([C.c_void_p, C.c_int, C.c_int, _I, _D, _I, _D, _D, _D, _I, _I] + [_D] * 16 +
                                       [_I])
    L.mbx_water_step_device.argtypes = [C.c_void_p, C.c_int, C.c_int, _D, C.c_int, C.c_int, _D] + \
        [C.c_void_p] * 19 + [_D]
    L.mbx_disp_list_builds.argtypes = [C.c_void_p]
    L.mbx_disp_list_builds.restype = C.c_long
    L.mbx_set_graphs.argtypes = [C.c_void_p, C.c_int]
    L.mbx_set_fused.argtypes = [C.c_void_p, C.c_int]
    L.mbx_set_fused_split.argtypes = [C.c_void_p, C.c_int]
    L.mbx_set_overlap.argtypes = [C.c_void_p, C.c_int, C.c_int]
    L.mbx_set_overlap_terms.argtypes = [C.c_void_p, C.c_int]
    L.mbx_set_final_fp64.argtypes = [C.c_void_p, C.c_int]
    L.mbx_graph_launches.argtypes = [C.c_void_p]
    L.mbx_graph_launches.restype = C.c_long
    L.mbx_last_lists.argtypes = [C.c_void_p, _I, C.c_long, _L, _I, C.c_long, _L]
    L.mbx_2b_poly_batch.argtypes = [C.c_void_p, C.c_int, C.c_long, _D, _D, _D, _D, _D]
    L.mbx_3b_poly_batch.argtypes = [C.c_void_p, C.c_int, C.c_long, _D, _D, _D, _D, _D, _D, _D]
    L.mbx_2b_force_matrix_batch.argtypes = [C.c_void_p, C.c_long, _D, _D, _D]
    L.mbx_3b_force_matrix_batch.argtypes = [C.c_void_p, C.c_long, _D, _D, _D, _D]
    L.mbx_pimd_matrices.argtypes = [C.c_int, C.c_int, _D, _D, _D]
    L.mbx_pimd_transform_device.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_long, C.c_void_p,
                                            C.c_void_p]
    L.mbx_pimd_spring_forces_device.argtypes = ([C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                                 C.c_double, C.c_int] + [C.c_void_p] * 7 + [_D])
    L.mbpol_2b_poly_.argtypes = [_D] * 6
    L.mbpol_2b_poly_.restype = None
    L.mbpol_3b_poly_.argtypes = [_D] * 8
    L.mbpol_3b_poly_.restype = None
    L.mbpol_2b_cutoff_.argtypes = [_D]
    L.mbpol_2b_cutoff_.restype = None
    L.mbpol_3b_cutoff_.argtypes = [_D]
    L.mbpol_3b_cutoff_.restype = None
    if path == LIB_PATH:
        _lib = L
    return L


def _p(a, t=_D):
    return None if a is None else a.ctypes.data_as(t)


def systems_polarizabilities(nw):
    from . import systems
    return systems.polarizabilities(nw)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Context:
    """One libmbx context (own CUDA stream and device buffers)."""

    def __init__(self, device=0):
        self.lib = load()
        h = C.c_void_p()
        rc = self.lib.mbx_create(C.byref(h), device)
        if rc:
            raise MbxError("mbx_create failed with status %d" % rc)
        self.h = h

    def close(self):
        if self.h:
            self.lib.mbx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc:
            raise MbxError("%s: status %d: %s" % (what, rc, self.lib.mbx_error(self.h).decode()))

    def set_stream(self, stream_ptr):
        self._check(self.lib.mbx_set_stream(self.h, C.c_void_p(stream_ptr)), "mbx_set_stream")

    def mbpol_forces(self, box, precision=FP64, heat=True, atomic_energy=True):
        """mbpol_forces on a WaterBox (host arrays).  Returns a dict like the oracle's."""
        n = box.natms
        x, y, z = (_f64(box.xyz[:, k]) for k in range(3))
        f = np.zeros((3, n))
        eng = C.c_double(0)
        vir = C.c_double(0)
        stress = np.zeros(9)
        ae = np.zeros(n) if atomic_energy else None
        sc = np.zeros(NSCALARS)
        v = [_f64(box.vel[:, k]) for k in range(3)] if heat else [None] * 3
        m = _f64(box.mass) if heat else None
        lst = np.ascontiguousarray(box.listttm2(), dtype=np.int32)
        rc = self.lib.mbx_mbpol_forces(self.h, precision, box.imcon, _p(_f64(box.cell)), 3 * box.nw, _p(lst, _I), n,
                                       _p(x), _p(y), _p(z), _p(f[0]), _p(f[1]), _p(f[2]), C.byref(eng),
                                       C.byref(vir), _p(stress), _p(v[0]), _p(v[1]), _p(v[2]), _p(m), _p(ae),
                                       _p(sc))
        self._check(rc, "mbx_mbpol_forces")
        out = dict(eng2=sc[S_ENG2], eng3=sc[S_ENG3], vir=sc[S_VIR], stress=sc[S_STRESS:S_STRESS + 9].copy(),
                   forces=f.T.copy(), atomic_energy=ae, jpot=sc[S_JPOT:S_JPOT + 3].copy(),
                   jkin=sc[S_JKIN:S_JKIN + 3].copy(), engsrp=eng.value, virsrp=vir.value, stress_acc=stress)
        return out

    def ps_pes(self, box, heat=True):
        """1-body PS PES over the box's H-O-H angles (host arrays)."""
        n = box.natms
        x, y, z = (_f64(box.xyz[:, k]) for k in range(3))
        f = np.zeros((3, n))
        eng = C.c_double(0)
        vir = C.c_double(0)
        stress = np.zeros(9)
        ae = np.zeros(n)
        jpot = np.zeros(3)
        v = [_f64(box.vel[:, k]) for k in range(3)] if heat else [None] * 3
        lst = np.ascontiguousarray(box.listang(), dtype=np.int32)
        rc = self.lib.mbx_ps_pes_forces(self.h, box.imcon, _p(_f64(box.cell)), box.nw, _p(lst, _I), n, _p(x), _p(y),
                                        _p(z), _p(f[0]), _p(f[1]), _p(f[2]), C.byref(eng), C.byref(vir), _p(stress),
                                        _p(v[0]), _p(v[1]), _p(v[2]), _p(ae), _p(jpot))
        self._check(rc, "mbx_ps_pes_forces")
        return dict(engang=eng.value, virang=vir.value, stress=stress, forces=f.T.copy(), atomic_energy=ae,
                    jpot=jpot)

    def msites_dms(self, box, gamma=0.426706882):
        """M sites and DMS charges (host arrays): (xyz with M sites, chge, dqdr[nw, 6])."""
        x, y, z = (_f64(box.xyz[:, k]).copy() for k in range(3))
        q = np.zeros(box.natms)
        dp = np.zeros((box.nw, 6))
        lst = np.ascontiguousarray(box.listttm2(), dtype=np.int32)
        self._check(self.lib.mbx_msites_dms(self.h, box.imcon, _p(_f64(box.cell)), 3 * box.nw, _p(lst, _I),
                                            box.natms, gamma, _p(x), _p(y), _p(z), _p(q), _p(dp)), "mbx_msites_dms")
        return np.stack([x, y, z], 1), q, dp

    def ps_pes_device(self, imcon, cell, nang, listang_ptr, natms, xyz_ptrs, f_ptrs, v_ptrs=None, ae_ptr=None):
        """Device-pointer 1-body PES; returns {engang, virang, stress[9], jpot[3]} as an array of 14."""
        out = np.zeros(14)
        v_ptrs = v_ptrs or (None, None, None)
        rc = self.lib.mbx_ps_pes_forces_device(self.h, imcon, _p(_f64(cell)), nang, listang_ptr, natms, *xyz_ptrs,
                                               *f_ptrs, *v_ptrs, ae_ptr, _p(out))
        self._check(rc, "mbx_ps_pes_forces_device")
        return out

    def mbpol_forces_device(self, precision, imcon, cell, nttm2, list_ptr, natms, xyz_ptrs, f_ptrs, v_ptrs=None,
                            mass_ptr=None, ae_ptr=None):
        """Device-pointer entry point (pointers as ints); returns the scalars."""
        sc = np.zeros(NSCALARS)
        v_ptrs = v_ptrs or (None, None, None)
        rc = self.lib.mbx_mbpol_forces_device(self.h, precision, imcon, _p(_f64(cell)), nttm2, list_ptr, natms,
                                              *xyz_ptrs, *f_ptrs, *v_ptrs, mass_ptr, ae_ptr, _p(sc))
        self._check(rc, "mbx_mbpol_forces_device")
        return sc

    def mbpol_multi(self, boxset, precision=FP64, heat=True, atomic_energy=True):
        """Every box of a BoxSet in one evaluation (host arrays).  Returns the packed
        forces/energies and scalars[nbox, NBOXSCALARS] (MB-pol block, then the 1-body
        engang, virang, stress[9], jpot[3])."""
        n = boxset.natms
        x, y, z = (_f64(boxset.xyz[:, k]) for k in range(3))
        f = np.zeros((3, n))
        ae = np.zeros(n) if atomic_energy else None
        sc = np.zeros((boxset.nbox, NBOXSCALARS))
        v = [_f64(boxset.vel[:, k]) for k in range(3)] if heat else [None] * 3
        m = _f64(boxset.mass) if heat else None
        nwb = np.ascontiguousarray(boxset.nw_box, dtype=np.int32)
        rc = self.lib.mbx_mbpol_multi(self.h, precision, boxset.imcon, boxset.nbox, _p(nwb, _I), _p(boxset.cells),
                                      _p(x), _p(y), _p(z), _p(f[0]), _p(f[1]), _p(f[2]), _p(v[0]), _p(v[1]),
                                      _p(v[2]), _p(m), _p(ae), _p(sc))
        self._check(rc, "mbx_mbpol_multi")
        return dict(forces=f.T.copy(), atomic_energy=ae, scalars=sc)

    def mbpol_multi_device(self, precision, boxset, xyz_ptrs, f_ptrs, v_ptrs=None, mass_ptr=None, ae_ptr=None,
                           cells=None):
        """Device-pointer multi-box entry point; returns scalars[nbox, NBOXSCALARS]."""
        sc = np.zeros((boxset.nbox, NBOXSCALARS))
        v_ptrs = v_ptrs or (None, None, None)
        nwb = np.ascontiguousarray(boxset.nw_box, dtype=np.int32)
        cells = boxset.cells if cells is None else _f64(cells)
        rc = self.lib.mbx_mbpol_multi_device(self.h, precision, boxset.imcon, boxset.nbox, _p(nwb, _I), _p(cells),
                                             *xyz_ptrs, *f_ptrs, *v_ptrs, mass_ptr, ae_ptr, _p(sc))
        self._check(rc, "mbx_mbpol_multi_device")
        return sc

    def water_forces(self, box, precision=FP64, heat=True, dispersion=False):
        """1-body + (dispersion) + MB-pol of one box in one call (host arrays)."""
        n = box.natms
        x, y, z = (_f64(box.xyz[:, k]) for k in range(3))
        f = np.zeros((3, n))
        ae = np.zeros(n)
        sc = np.zeros(NWATERSCALARS)
        v = [_f64(box.vel[:, k]) for k in range(3)] if heat else [None] * 3
        m = _f64(box.mass) if heat else None
        lst = np.ascontiguousarray(box.listttm2(), dtype=np.int32)
        ang = np.ascontiguousarray(box.listang(), dtype=np.int32)
        lt = mo = None
        if dispersion:
            from mbx import systems
            lt, mo = systems.water_types(box)
        rc = self.lib.mbx_water_forces(self.h, precision, box.imcon, _p(_f64(box.cell)), 3 * box.nw, _p(lst, _I),
                                       box.nw, _p(ang, _I), _p(lt, _I), _p(mo, _I), n, _p(x), _p(y), _p(z),
                                       _p(f[0]), _p(f[1]), _p(f[2]), _p(v[0]), _p(v[1]), _p(v[2]), _p(m), _p(ae),
                                       _p(sc))
        self._check(rc, "mbx_water_forces")
        return dict(forces=f.T.copy(), atomic_energy=ae, scalars=sc)

    def disp_setup(self, prm, rcut=9.0, delr=1.0, mxgrid=0, ntypes=None):
        prm = _f64(prm).reshape(-1, 4)
        nt = ntypes or int(round((np.sqrt(8 * prm.shape[0] + 1) - 1) / 2))
        self._check(self.lib.mbx_disp_setup(self.h, nt, _p(prm.ravel().copy()), rcut, delr, mxgrid),
                    "mbx_disp_setup")

    def dispersion(self, box, ltype, mol, heat=True):
        """Dispersion forces on a box (host arrays); ltype/mol per atom."""
        n = box.natms
        x, y, z = (_f64(box.xyz[:, k]) for k in range(3))
        f = np.zeros((3, n))
        eng = C.c_double(0)
        vir = C.c_double(0)
        stress = np.zeros(9)
        ae = np.zeros(n)
        jpot = np.zeros(3)
        v = [_f64(box.vel[:, k]) for k in range(3)] if heat else [None] * 3
        lt = np.ascontiguousarray(ltype, dtype=np.int32)
        mo = np.ascontiguousarray(mol, dtype=np.int32)
        rc = self.lib.mbx_disp_forces(self.h, box.imcon, _p(_f64(box.cell)), n, _p(lt, _I), _p(mo, _I), _p(x),
                                      _p(y), _p(z), _p(f[0]), _p(f[1]), _p(f[2]), C.byref(eng), C.byref(vir),
                                      _p(stress), _p(v[0]), _p(v[1]), _p(v[2]), _p(ae), _p(jpot))
        self._check(rc, "mbx_disp_forces")
        return dict(eng=eng.value, vir=vir.value, stress=stress, forces=f.T.copy(), atomic_energy=ae, jpot=jpot)

    def polar(self, sites, cell, imcon, nw, chge, dp, polr, polr2, prm, dip0=None, vel=None, atomic_energy=True,
              check=True, precision=FP64):
        """TTM4-F electrostatics (mbx_polar_forces, host arrays) on 4*nw sites; returns a
        dict shaped like the oracle's."""
        n = 4 * nw
        x, y, z = (_f64(sites[:, k]) for k in range(3))
        dip = np.zeros((3, n)) if dip0 is None else np.ascontiguousarray(np.asarray(dip0, np.float64).T).copy()
        f = np.zeros((3, n))
        out = np.zeros(16)
        ae = np.zeros(n) if atomic_energy else None
        jpot = np.zeros(3)
        jkin = np.zeros(3)
        v = [_f64(vel[:3 * nw, k]) for k in range(3)] if vel is not None else [None] * 3
        rc = self.lib.mbx_polar_forces(self.h, precision, _p(_f64(prm)), imcon, _p(_f64(cell)), nw, _p(x), _p(y), _p(z),
                                       _p(_f64(chge)), _p(_f64(dp)), _p(_f64(polr)), _p(_f64(polr2)), _p(dip[0]),
                                       _p(dip[1]), _p(dip[2]), _p(f[0]), _p(f[1]), _p(f[2]), _p(out), _p(ae),
                                       _p(v[0]), _p(v[1]), _p(v[2]), _p(jpot), _p(jkin))
        if check:
            self._check(rc, "mbx_polar_forces")
        return dict(status=rc, forces=f.T.copy(), engcpe=out[0], vircpe=out[1], stress=out[2:11].copy(),
                    iterations=int(out[11]), deltadip=out[12], eng_polar=out[13], eng_kspace=out[14],
                    eng_real=out[15], dipoles=dip.T.copy(), atomic_energy=ae, jpot=jpot, jkin=jkin)

    def water_step(self, box, polar_prm, precision=MIXED, dip0=None, disp=None, heat=True, check=True):
        """mbx_water_step on a WaterBox (standard layout): the whole force evaluation of one
        MD step.  disp = (ltype, mol) after disp_setup, or None.  Returns a dict."""
        n = box.natms
        x, y, z = (_f64(box.xyz[:, k]).copy() for k in range(3))
        dip = np.zeros((3, n)) if dip0 is None else np.ascontiguousarray(np.asarray(dip0, np.float64).T).copy()
        f = np.zeros((3, n))
        ae = np.zeros(n)
        q = np.zeros(n)
        sc = np.zeros(NSTEPSCALARS)
        polr, polr2 = systems_polarizabilities(box.nw)
        v = [_f64(box.vel[:, k]) for k in range(3)] if heat else [None] * 3
        m = _f64(box.mass) if heat else None
        lt, mo = (None, None) if disp is None else (np.ascontiguousarray(disp[0], np.int32),
                                                    np.ascontiguousarray(disp[1], np.int32))
        rc = self.lib.mbx_water_step(self.h, precision, box.imcon, _p(_f64(box.cell)), box.nw, n,
                                     _p(_f64(polar_prm)), _p(polr), _p(polr2), _p(lt, _I), _p(mo, _I), _p(x), _p(y),
                                     _p(z), _p(dip[0]), _p(dip[1]), _p(dip[2]), _p(f[0]), _p(f[1]), _p(f[2]),
                                     _p(v[0]), _p(v[1]), _p(v[2]), _p(m), _p(ae), _p(q), _p(sc))
        if check:
            self._check(rc, "mbx_water_step")
        return dict(status=rc, forces=f.T.copy(), atomic_energy=ae, chge=q, scalars=sc, dipoles=dip.T.copy(),
                    sites=np.stack([x, y, z], 1))

    def ipi_run(self, address, precision=MIXED, polar_prm=None, dispersion=False, max_steps=0):
        """mbx_ipi_run: i-PI driver mode on this context; returns the force replies sent"""
        steps = C.c_long(0)
        prm = None if polar_prm is None else _f64(polar_prm)
        rc = self.lib.mbx_ipi_run(self.h, address.encode(), precision, _p(prm), 1 if dispersion else 0,
                                  int(max_steps), C.byref(steps))
        self._check(rc, "mbx_ipi_run")
        return int(steps.value)

    def set_precond_block(self, on):
        """Per-water block-Jacobi preconditioner of the mixed dipole solve (on by default;
        off: the sweeps of set_precond_sweeps)."""
        self._check(self.lib.mbx_set_precond_block(self.h, int(bool(on))), "mbx_set_precond_block")

    def set_precond_sweeps(self, sweeps):
        self._check(self.lib.mbx_set_precond_sweeps(self.h, int(sweeps)), "mbx_set_precond_sweeps")

    def set_aspc(self, k, iter_nstep=None):
        """ASPC dipole prediction of order k (2 or 4; 0: off) after iter_nstep converged
        steps (default k+2); clears the history and the step count."""
        n = (int(k) + 2 if k else 0) if iter_nstep is None else int(iter_nstep)
        self._check(self.lib.mbx_set_aspc(self.h, int(k), n), "mbx_set_aspc")

    def set_dipole_guess(self, order):
        """Extrapolated initial guess of the converged dipole solves (order 1..3; 0 off);
        clears the history."""
        self._check(self.lib.mbx_set_dipole_guess(self.h, int(order)), "mbx_set_dipole_guess")

    def aspc_restart(self):
        self._check(self.lib.mbx_aspc_restart(self.h), "mbx_aspc_restart")

    def aspc_step(self):
        return int(self.lib.mbx_aspc_step(self.h))

    def set_spme(self, order=6, spacing=0.8, grid=None):
        """k space of later electrostatics calls: SPME of `order` (0: the Ewald sum) on
        `grid` (3 ints) or the grid of `spacing`."""
        g = None if grid is None else np.ascontiguousarray(grid, np.int32)
        self._check(self.lib.mbx_set_spme(self.h, int(order), float(spacing), _p(g, _I)), "mbx_set_spme")

    def set_polar_skin(self, delr):
        self._check(self.lib.mbx_set_polar_skin(self.h, float(delr)), "mbx_set_polar_skin")

    def polar_list_builds(self):
        return int(self.lib.mbx_polar_list_builds(self.h))

    def polar_last_pairs(self):
        """(npairs x 2) site pairs i < j within rcut of the last electrostatics call"""
        n = C.c_long(0)
        self._check(self.lib.mbx_polar_last_pairs(self.h, None, 0, C.byref(n)), "mbx_polar_last_pairs")
        out = np.zeros((max(n.value, 1), 2), np.int32)
        self._check(self.lib.mbx_polar_last_pairs(self.h, _p(out, _I), n.value, C.byref(n)), "mbx_polar_last_pairs")
        return out[:n.value]

    def spme_last_grid(self):
        g = np.zeros(3, np.int32)
        self._check(self.lib.mbx_spme_last_grid(self.h, _p(g, _I)), "mbx_spme_last_grid")
        return tuple(int(v) for v in g)

    def spme_kspace(self, sites, cell, imcon, chge, alpha, grid, order=6, dip=None, vel=None, epsq=1.0):
        """mbx_spme_kspace on host arrays: sites (n x 3), chge (n), dip / vel (n x 3) or None.
        Returns dict(engc, eng, stress (9), jpot (3), forces, field, pot)."""
        sites = np.asarray(sites, np.float64)
        n = sites.shape[0]
        x, y, z = (_f64(sites[:, k]) for k in range(3))
        d = None if dip is None else np.ascontiguousarray(np.asarray(dip, np.float64).T).reshape(-1)
        v = None if vel is None else np.ascontiguousarray(np.asarray(vel, np.float64).T).reshape(-1)
        f = np.zeros(3 * n)
        fld = np.zeros(3 * n)
        pot = np.zeros(n)
        out = np.zeros(14)
        prm = np.array([alpha, epsq], np.float64)
        g = np.ascontiguousarray(grid, np.int32)
        rc = self.lib.mbx_spme_kspace(self.h, _p(prm), int(order), _p(g, _I), int(imcon), _p(_f64(cell)), n, _p(x),
                                      _p(y), _p(z), _p(_f64(chge)), _p(d), _p(v), _p(f), _p(fld), _p(pot), _p(out))
        self._check(rc, "mbx_spme_kspace")
        return dict(engc=out[0], eng=out[1], stress=out[2:11].copy(), jpot=out[11:14].copy(),
                    forces=f.reshape(3, n).T.copy(), field=fld.reshape(3, n).T.copy(), pot=pot)

    def fft3d(self, data, sign=1):
        """mbx_fft3d on a complex array of shape (count, n3, n2, n1) or (n3, n2, n1) (x fastest)."""
        a = np.ascontiguousarray(data, np.complex128)
        shp = a.shape
        if a.ndim == 3:
            a = a[None]
        cnt, n3, n2, n1 = a.shape
        buf = np.ascontiguousarray(a).view(np.float64).reshape(-1).copy()
        self._check(self.lib.mbx_fft3d(self.h, n1, n2, n3, cnt, int(sign), _p(buf)), "mbx_fft3d")
        return buf.view(np.complex128).reshape(shp)

    def set_lanes(self, lanes):
        self._check(self.lib.mbx_set_lanes(self.h, int(lanes)), "mbx_set_lanes")

    def water_step_multi(self, boxes, polar_prms, precision=MIXED, dip0=None, disp=None, heat=True, check=True):
        """mbx_water_step_multi on a list of WaterBoxes (standard layout), polar_prms one
        15-vector per box; dip0 (sites x 3, all boxes concatenated) or None; disp = (ltype,
        mol) concatenated, after disp_setup.  Returns a dict with per-box scalars and status."""
        nb = len(boxes)
        nws = np.array([b.nw for b in boxes], np.int32)
        imc = np.array([b.imcon for b in boxes], np.int32)
        cells = np.concatenate([_f64(b.cell) for b in boxes]) if nb else np.zeros(9)
        prm = np.ascontiguousarray(np.concatenate([_f64(p) for p in polar_prms]) if nb else np.zeros(15))
        xyz = np.concatenate([b.xyz for b in boxes]) if nb else np.zeros((0, 3))
        n = xyz.shape[0]
        x, y, z = (np.ascontiguousarray(xyz[:, k], np.float64).copy() for k in range(3))
        dip = np.zeros((3, n)) if dip0 is None else np.ascontiguousarray(np.asarray(dip0, np.float64).T).copy()
        f = np.zeros((3, n))
        ae = np.zeros(n)
        q = np.zeros(n)
        sc = np.zeros((max(nb, 1), NSTEPSCALARS))
        st = np.zeros(max(nb, 1), np.int32)
        pol = [systems_polarizabilities(b.nw) for b in boxes]
        polr = np.concatenate([p[0] for p in pol]) if nb else np.zeros(1)
        polr2 = np.concatenate([p[1] for p in pol]) if nb else np.zeros(1)
        if heat and nb:
            vel = np.concatenate([b.vel for b in boxes])
            v = [np.ascontiguousarray(vel[:, k], np.float64) for k in range(3)]
            m = np.ascontiguousarray(np.concatenate([b.mass for b in boxes]), np.float64)
        else:
            v, m = [None] * 3, None
        lt, mo = (None, None) if disp is None or not nb else (np.ascontiguousarray(disp[0], np.int32),
                                                              np.ascontiguousarray(disp[1], np.int32))
        rc = self.lib.mbx_water_step_multi(self.h, precision, nb, _p(imc, _I), _p(cells), _p(nws, _I), _p(prm),
                                           _p(polr), _p(polr2), _p(lt, _I), _p(mo, _I), _p(x), _p(y), _p(z),
                                           _p(dip[0]), _p(dip[1]), _p(dip[2]), _p(f[0]), _p(f[1]), _p(f[2]),
                                           _p(v[0]), _p(v[1]), _p(v[2]), _p(m), _p(ae), _p(q), _p(sc), _p(st, _I))
        if check:
            self._check(rc, "mbx_water_step_multi")
        return dict(status=rc, box_status=st[:nb].copy(), forces=f.T.copy(), atomic_energy=ae, chge=q,
                    scalars=sc[:nb].copy(), dipoles=dip.T.copy(), sites=np.stack([x, y, z], 1))

    def polar_iterations(self):
        return int(self.lib.mbx_polar_iterations(self.h))

    def polar_timings(self):
        """(ms[4]: setup, dipole solve, final structure factors, rest of the final pass; K)"""
        ms = (C.c_float * 4)()
        kv = C.c_long(0)
        self._check(self.lib.mbx_polar_timings(self.h, ms, C.byref(kv)), "mbx_polar_timings")
        return np.array(list(ms)), int(kv.value)

    def polar_field_timing(self):
        """(ms, algorithmic flops, launches) of the last call's FP64 k-space field gathers"""
        ms = np.zeros(1)
        fl = np.zeros(1)
        n = C.c_long(0)
        self._check(self.lib.mbx_polar_field_timing(self.h, _p(ms), _p(fl), C.byref(n)), "mbx_polar_field_timing")
        return float(ms[0]), float(fl[0]), int(n.value)

    def polar_inner_sweeps(self):
        return int(self.lib.mbx_polar_inner_sweeps(self.h))

    def disp_list_builds(self):
        return int(self.lib.mbx_disp_list_builds(self.h))

    def set_fused(self, on=True):
        self._check(self.lib.mbx_set_fused(self.h, 1 if on else 0), "mbx_set_fused")

    def set_overlap_terms(self, on):
        """1-body and dispersion terms on a third stream beside the electrostatics (on/off)."""
        self._check(self.lib.mbx_set_overlap_terms(self.h, int(bool(on))), "mbx_set_overlap_terms")

    def set_final_fp64(self, on):
        """Mixed method: the electrostatics' final pass in FP64 (on/off); the solve stays mixed."""
        self._check(self.lib.mbx_set_final_fp64(self.h, int(bool(on))), "mbx_set_final_fp64")

    def set_overlap(self, on=True, dimer_warps=0):
        """The MB-pol terms beside the electrostatics' dipole solve in mbx_water_step (mixed)."""
        self._check(self.lib.mbx_set_overlap(self.h, 1 if on else 0, int(dimer_warps)), "mbx_set_overlap")

    def set_fused_split(self, dimer_warps=0):
        """Dimer warps of the fused 2B/3B kernel's 12 per block (0: the default, 4)."""
        self._check(self.lib.mbx_set_fused_split(self.h, int(dimer_warps)), "mbx_set_fused_split")

    def set_graphs(self, on=True):
        self._check(self.lib.mbx_set_graphs(self.h, 1 if on else 0), "mbx_set_graphs")

    def graph_launches(self):
        return int(self.lib.mbx_graph_launches(self.h))

    def set_profiling(self, on=True):
        self._check(self.lib.mbx_set_profiling(self.h, 1 if on else 0), "mbx_set_profiling")

    def last_timings(self):
        """(phase ms [lists, 2B, 3B, jkin], (dimers, trimers, launches, hard dimers, hard trimers))"""
        ms = np.zeros(4)
        cnt = (C.c_long * 5)()
        self._check(self.lib.mbx_last_timings(self.h, _p(ms), cnt), "mbx_last_timings")
        return ms, tuple(cnt[q] for q in range(5))

    def set_mixed_limits(self, limit2b, limit3b):
        self._check(self.lib.mbx_set_mixed_limits(self.h, limit2b, limit3b), "mbx_set_mixed_limits")

    def last_lists(self):
        npairs = C.c_long(0)
        ntrip = C.c_long(0)
        self._check(self.lib.mbx_last_lists(self.h, None, 0, C.byref(npairs), None, 0, C.byref(ntrip)),
                    "mbx_last_lists")
        pairs = np.zeros(2 * max(npairs.value, 1), np.int32)
        trip = np.zeros(3 * max(ntrip.value, 1), np.int32)
        self._check(self.lib.mbx_last_lists(self.h, _p(pairs, _I), npairs.value, C.byref(npairs), _p(trip, _I),
                                            ntrip.value, C.byref(ntrip)), "mbx_last_lists")
        return pairs[:2 * npairs.value].reshape(-1, 2), trip[:3 * ntrip.value].reshape(-1, 3)

    def poly2b_batch(self, W1, W2, precision=FP64):
        W1 = _f64(W1).reshape(-1, 9)
        W2 = _f64(W2).reshape(-1, 9)
        n = W1.shape[0]
        E = np.zeros(n)
        g1 = np.zeros((n, 9))
        g2 = np.zeros((n, 9))
        self._check(self.lib.mbx_2b_poly_batch(self.h, precision, n, _p(W1), _p(W2), _p(E), _p(g1), _p(g2)),
                    "mbx_2b_poly_batch")
        return E, g1, g2

    def poly3b_batch(self, W1, W2, W3, precision=FP64, g=None):
        W = [_f64(w).reshape(-1, 9) for w in (W1, W2, W3)]
        n = W[0].shape[0]
        E = np.zeros(n)
        gs = [np.zeros((n, 9)) for _ in range(3)] if g is None else [_f64(a).reshape(-1, 9).copy() for a in g]
        self._check(self.lib.mbx_3b_poly_batch(self.h, precision, n, *(_p(w) for w in W), _p(E),
                                               *(_p(a) for a in gs)), "mbx_3b_poly_batch")
        return (E, *gs)


class Server:
    """Continuous-batching force server (mbx_server_*): concurrent independent boxes."""

    def __init__(self, device=0, slots=4, budget_bytes=32e9):
        self.lib = load()
        h = C.c_void_p()
        rc = self.lib.mbx_server_create(C.byref(h), device, slots, float(budget_bytes))
        if rc:
            raise MbxError("mbx_server_create failed with status %d" % rc)
        self.h = h
        self._boxes = {}

    def set_spme(self, order=6, spacing=0.8):
        """k space of later step requests: SPME (order 4..8) or the Ewald sum (order 0)."""
        rc = self.lib.mbx_server_set_spme(self.h, int(order), float(spacing))
        if rc:
            raise MbxError("mbx_server_set_spme failed with status %d" % rc)

    def close(self):
        if self.h:
            self.lib.mbx_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, box, precision=MIXED, heat=True):
        x, y, z = (_f64(box.xyz[:, k]) for k in range(3))
        v = [_f64(box.vel[:, k]) for k in range(3)] if heat else [None] * 3
        m = _f64(box.mass) if heat else None
        rid = self.lib.mbx_server_submit(self.h, precision, box.imcon, _p(_f64(box.cell)), box.nw, box.natms,
                                         _p(x), _p(y), _p(z), _p(v[0]), _p(v[1]), _p(v[2]), _p(m))
        if rid <= 0:
            raise MbxError("mbx_server_submit failed with status %d" % -rid)
        self._boxes[rid] = box.natms
        return rid

    def wait(self, rid):
        n = self._boxes.pop(rid)
        f = np.zeros((3, n))
        ae = np.zeros(n)
        sc = np.zeros(NSCALARS + 14)
        t = np.zeros(3)
        rc = self.lib.mbx_server_wait(self.h, rid, _p(f[0]), _p(f[1]), _p(f[2]), _p(ae), _p(sc), _p(t))
        if rc:
            raise MbxError("request %d failed with status %d" % (rid, rc))
        return dict(forces=f.T.copy(), atomic_energy=ae, scalars=sc, queue_s=t[0], run_s=t[1], latency_s=t[2])

    def submit_step(self, box, client, precision=MIXED, heat=True):
        """The whole force evaluation with the electrostatics; dipoles warm-started from the
        client's previous request."""
        x, y, z = (_f64(box.xyz[:, k]) for k in range(3))
        v = [_f64(box.vel[:, k]) for k in range(3)] if heat else [None] * 3
        m = _f64(box.mass) if heat else None
        rid = self.lib.mbx_server_submit_step(self.h, precision, int(client), box.imcon, _p(_f64(box.cell)), box.nw,
                                              _p(x), _p(y), _p(z), _p(v[0]), _p(v[1]), _p(v[2]), _p(m))
        if rid <= 0:
            raise MbxError("mbx_server_submit_step failed with status %d" % -rid)
        self._boxes[rid] = box.natms
        return rid

    def wait_step(self, rid):
        n = self._boxes.pop(rid)
        f = np.zeros((3, n))
        ae = np.zeros(n)
        dip = np.zeros((3, n))
        sc = np.zeros(NSTEPSCALARS)
        t = np.zeros(3)
        rc = self.lib.mbx_server_wait_step(self.h, rid, _p(f[0]), _p(f[1]), _p(f[2]), _p(ae), _p(dip.reshape(-1)),
                                           _p(sc), _p(t))
        if rc:
            raise MbxError("request %d failed with status %d: %s" % (rid, rc, self.lib.mbx_server_error(self.h).decode()))
        return dict(forces=f.T.copy(), atomic_energy=ae, dipoles=dip.T.copy(), scalars=sc, queue_s=t[0],
                    run_s=t[1], latency_s=t[2])
