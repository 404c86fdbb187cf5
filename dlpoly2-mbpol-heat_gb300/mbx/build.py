"""Build libmbx.so (sm_103a) in-tree, and the CPU oracle used by the tests.

Steps: generate the polynomial PTX modules from the committed monomial tables,
compile every PTX module and CUDA source as relocatable device code in parallel,
then device-link everything into one shared library.  Outputs go to
``<package>/_build`` (git-ignored).  Nothing here needs a GPU.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REPO = os.path.dirname(PKG)
BUILD = os.path.join(PKG, "_build")
CSRC = os.path.join(PKG, "csrc")
LIB = os.path.join(BUILD, "libmbx.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SOURCES = ["mbx_lists.cu", "mbx_mbpol.cu", "mbx_capi.cu", "mbx_noalloc.cu", "mbx_pes.cu", "mbx_server.cu",
                "mbx_multi.cu", "mbx_disp.cu", "mbx_polar.cu", "mbx_ipi.cu", "mbx_spme.cu", "mbx_pimd.cu"]
HEADERS = ["mbx_common.cuh", "mbx_kernels.cuh", "mbx_spme.cuh"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def _stale(target, deps, cmd):
    """Rebuild when a dependency is newer or the command line changed."""
    rec = target + ".cmd"
    line = " ".join(cmd)
    if _newer(target, deps) or not os.path.exists(rec):
        return True
    with open(rec) as f:
        return f.read() != line


def _compile(cmd, target):
    out = _run(cmd)
    with open(target + ".cmd", "w") as f:
        f.write(" ".join(cmd))
    return out


def _check_stamp():
    """Objects from another machine (x86 here, aarch64 on the GPU hosts) are discarded."""
    import platform
    stamp = os.path.join(BUILD, "PLATFORM")
    me = platform.machine() + " " + _run([_nvcc(), "--version"]).strip().splitlines()[-1]
    if os.path.isdir(BUILD):
        old = open(stamp).read() if os.path.exists(stamp) else ""
        if old != me:
            shutil.rmtree(BUILD)
    os.makedirs(BUILD, exist_ok=True)
    with open(stamp, "w") as f:
        f.write(me)


# Register budget of the generated polynomial functions.  The fused mixed-precision
# kernel (12 warps per SM: 4 on FP64 dimers, 8 on FP32 trimers) runs at 168 registers,
# so every function it calls -- the FP64 2B and the FP32 chunks -- is compiled within
# that budget.  The FP64 3B chunks serve only the separate FP64 3B kernel and keep the
# full register file.
FUSED_MAXRREG = 168


def _poly_reg_flags(ptx_path):
    name = os.path.basename(ptx_path)
    if "poly3b_f64" in name or "coef" in name:
        return []
    return ["-maxrregcount=%d" % FUSED_MAXRREG]


def build_lib(verbose=False, jobs=None):
    _check_stamp()
    sys.path.insert(0, os.path.join(PKG, "gen"))
    import gen_poly_ptx  # noqa: E402

    gen_dir = os.path.join(BUILD, "gen")
    os.makedirs(gen_dir, exist_ok=True)
    ptx = gen_poly_ptx.generate(os.path.join(PKG, "tables"), gen_dir)
    import gen_pes  # noqa: E402
    gen_pes.generate(os.path.join(PKG, "tables"), gen_dir)
    nvcc = _nvcc()
    common = ARCH + ["-Xcompiler", "-fPIC", "-rdc=true"]
    jobs_list = []
    for p in ptx:
        o = p[:-4] + ".o"
        cmd = [nvcc] + common + _poly_reg_flags(p) + ["-c", p, "-o", o]
        if _stale(o, [p], cmd):
            jobs_list.append((o, cmd))
    hdr_deps = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(gen_dir, "mbx_poly_gen.cuh"),
                                                          os.path.join(gen_dir, "mbx_pes_gen.cuh"),
                                                          os.path.join(REPO, "include", "mbx.h")]
    cu_objs = []
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        cu_objs.append(o)
        cmd = [nvcc] + common + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-I", CSRC, "-I",
                                 gen_dir, "-c", s, "-o", o]
        if _stale(o, [s] + hdr_deps, cmd):
            jobs_list.append((o, cmd))
    jobs = jobs or max(2, os.cpu_count() or 2)
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        outs = list(ex.map(lambda j: _compile(j[1], j[0]), jobs_list))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    objs = cu_objs + [p[:-4] + ".o" for p in ptx]
    if _newer(LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-rdc=true", "-Xcompiler", "-fPIC", "-o", LIB] + objs)
    return LIB


def build_oracle(reference_source=None):
    """Compile the oracle, and the reference's own C++ polynomials when the path of the
    reference's SOURCE directory is given (argument, else the environment variable
    MBX_REFERENCE_SOURCE); without one only the oracle is built."""
    odir = os.path.join(REPO, "oracle")
    _run(["make", "-s", "-B", "-C", odir, "liboracle.so"])
    ref = reference_source or os.environ.get("MBX_REFERENCE_SOURCE")
    if ref and os.path.isdir(ref):
        _run(["make", "-s", "-C", odir, "ref", "REFSRC=" + ref])
    return os.path.join(odir, "liboracle.so")


if __name__ == "__main__":
    print(build_lib(verbose=True))
    print(build_oracle())
