"""Build recipe for the native parts of noa_gb300 (no cmake).

    python -m noa_gb300.build            # CUDA library + CPU oracle
    python -m noa_gb300.build --ref      # also the reference's own code (oracle/build_ref.sh)

Products (all git-ignored, built in place):
    noa_gb300/libnoa_dcs.so      CUDA kernels + C ABI of include/noa_dcs.h, sm_103a only
    noa_gb300/libnoa_dcs_torch.so  LibTorch drop-in (include/noa_gb300/dcs_cuda.hh)
    noa_gb300/libnoa_dcs_diag.so   test / bench instruments (csrc/diag/noa_dcs_diag.h), not the product
    noa_gb300/_muons_cuda*.so    Python module mirroring the reference notebook's extension
    oracle/liboracle_dcs.so      CPU restatement of the reference, the tests' oracle
    oracle/_ref/libnoa_ref_dcs.so  the reference's own dcs.hh on the CPU
    oracle/_ref/libnoa_ref_cuda.so the reference's own CUDA bremsstrahlung kernel
    oracle/_ref/ref_dropin_caller  a reference-side program linked with libnoa_dcs_torch.so
                                   (the three oracle/_ref products only where a noa checkout
                                   or its staged headers exist; oracle/build_ref.sh)

Each .cu file is compiled in its own nvcc process, in parallel, then linked.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libnoa_dcs.so")
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "liboracle_dcs.so")
REF_LIB = os.path.join(ORACLE_DIR, "_ref", "libnoa_ref_dcs.so")
REF_CUDA_LIB = os.path.join(ORACLE_DIR, "_ref", "libnoa_ref_cuda.so")
REF_CALLER = os.path.join(ORACLE_DIR, "_ref", "ref_dropin_caller")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr",
                     "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", os.path.join(ROOT, "include")]


# Per-file extra flags.  coulomb.cu keeps the reference's IEEE operation
# order (no FMA contraction): its Ridders iteration branches on signs of
# differences, so contraction could change the iteration path.
FILE_FLAGS = {"coulomb.cu": ["-fmad=false"]}


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed:\n  " + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs + [os.path.join(ROOT, "include", "noa_dcs.h")]


DIAG_DIR = os.path.join(CSRC, "diag")
DIAG_LIB = os.path.join(PKG, "libnoa_dcs_diag.so")


def build_diag():
    """libnoa_dcs_diag.so: the test and bench instruments (FMA-chain peak
    probe, element-wise evaluator of the library's elementary functions),
    kept out of the product library libnoa_dcs.so."""
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(os.path.join(DIAG_DIR, f) for f in os.listdir(DIAG_DIR) if f.endswith(".cu"))
    deps = _headers() + [os.path.join(DIAG_DIR, "noa_dcs_diag.h")]
    objs = [os.path.join(BUILD, "diag_" + os.path.basename(s)[:-3] + ".o") for s in srcs]
    jobs = [(s, o) for s, o in zip(srcs, objs) if _stale(o, [s] + deps)]
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(lambda so: _run([nvcc] + NVCC_FLAGS + ["-c", so[0], "-o", so[1]]), jobs))
    if jobs or _stale(DIAG_LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", DIAG_LIB] + objs)
    return DIAG_LIB


def build_cuda(verbose=False):
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    hdrs = _headers()
    objs = [os.path.join(BUILD, os.path.basename(s)[:-3] + ".o") for s in srcs]
    jobs = [(s, o) for s, o in zip(srcs, objs) if _stale(o, [s] + hdrs)]
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        outs = list(ex.map(lambda so: _run([nvcc] + NVCC_FLAGS + FILE_FLAGS.get(os.path.basename(so[0]), []) +
                                           ["-c", so[0], "-o", so[1]]), jobs))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    if jobs or _stale(LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcuda"])
    return LIB


TORCH_LIB = os.path.join(PKG, "libnoa_dcs_torch.so")


def _torch_flags():
    import sysconfig
    import torch
    tdir = os.path.dirname(torch.__file__)
    abi = int(bool(torch._C._GLIBCXX_USE_CXX11_ABI))
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(_nvcc())), "include")
    inc = ["-I", os.path.join(ROOT, "include"), "-I", os.path.join(tdir, "include"),
           "-I", os.path.join(tdir, "include", "torch", "csrc", "api", "include"), "-I", cuda_inc,
           "-I", sysconfig.get_paths()["include"]]
    cflags = ["-std=c++17", "-O2", "-fPIC", f"-D_GLIBCXX_USE_CXX11_ABI={abi}"] + inc
    libs = ["-L", os.path.join(tdir, "lib"), f"-Wl,-rpath,{os.path.join(tdir, 'lib')}", "-Wl,-rpath,$ORIGIN",
            "-ltorch", "-ltorch_cpu", "-lc10", "-lc10_cuda", "-ltorch_cuda"]
    return cflags, libs


def compile_torch_objects():
    """Compiles the two LibTorch translation units (the slow part) in parallel."""
    cflags, _ = _torch_flags()
    src_dir = os.path.join(CSRC, "torch")
    hdr = os.path.join(ROOT, "include", "noa_gb300", "dcs_cuda.hh")
    os.makedirs(BUILD, exist_ok=True)
    jobs = []
    for name, extra in (("dcs_cuda", []),
                        ("muons_cuda", ["-DTORCH_EXTENSION_NAME=_muons_cuda", "-DTORCH_API_INCLUDE_EXTENSION_H"])):
        src = os.path.join(src_dir, name + ".cpp")
        obj = os.path.join(BUILD, name + ".torch.o")
        if _stale(obj, [src, hdr, os.path.join(ROOT, "include", "noa_dcs.h")]):
            jobs.append(["g++"] + cflags + extra + ["-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        list(ex.map(_run, jobs))
    return [os.path.join(BUILD, n + ".torch.o") for n in ("dcs_cuda", "muons_cuda")]


def build_torch(objs=None):
    """LibTorch drop-in (libnoa_dcs_torch.so, the noa::pms::dcs::cuda symbols)
    and the Python module _muons_cuda that mirrors the reference notebook's
    muons_cuda extension.  Needs libnoa_dcs.so built first."""
    import sysconfig
    _, libs = _torch_flags()
    o_dropin, o_mod = objs or compile_torch_objects()
    if _stale(TORCH_LIB, [o_dropin, LIB]):
        _run(["g++", "-shared", o_dropin, "-o", TORCH_LIB, "-L", PKG, "-lnoa_dcs"] + libs)
    ext = os.path.join(PKG, "_muons_cuda" + sysconfig.get_config_var("EXT_SUFFIX"))
    if _stale(ext, [o_mod, TORCH_LIB]):
        _run(["g++", "-shared", o_mod, "-o", ext, "-L", PKG, "-lnoa_dcs_torch", "-lnoa_dcs"] + libs +
             ["-ltorch_python"])
    return TORCH_LIB, ext


def build_oracle():
    src = os.path.join(ORACLE_DIR, "dcs_oracle.cpp")
    hdr = os.path.join(ORACLE_DIR, "dcs_oracle.hpp")
    if _stale(ORACLE_LIB, [src, hdr]):
        _run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC",
              "-shared", src, "-o", ORACLE_LIB])
    return ORACLE_LIB


def build_ref(stage="all"):
    """Builds the reference's own code with oracle/build_ref.sh (test and bench
    infrastructure): stage "all" gives oracle/_ref/libnoa_ref_dcs.so (the
    reference's CPU dcs::vmap / dcs::pvmap) and oracle/_ref/libnoa_ref_cuda.so
    (its CUDA bremsstrahlung kernel); stage "caller" gives
    oracle/_ref/ref_dropin_caller, linked with libnoa_dcs_torch.so.  The
    script reads a noa checkout (NOA_CHECKOUT) or the copy of its headers
    staged in oracle/_ref/src; with neither it does nothing and this returns
    None.  A failure is recorded in oracle/_ref/build_<stage>.log and returns None:
    the reference's code is a checker and a baseline, never a product
    dependency, so it must not stop the product's build."""
    log = os.path.join(ORACLE_DIR, "_ref", f"build_{stage}.log")
    try:
        text = _run(["bash", os.path.join(ORACLE_DIR, "build_ref.sh"), stage])
    except RuntimeError as e:
        text = str(e)
        ok = False
    else:
        ok = True
    if os.path.isdir(os.path.dirname(log)):
        with open(log, "w") as f:
            f.write(("ok\n" if ok else "FAILED\n") + text)
    target = {"all": REF_LIB, "caller": REF_CALLER}[stage]
    return target if ok and os.path.exists(target) else None


def build_all(ref=True, torch_layer=True, verbose=False):
    with cf.ThreadPoolExecutor(max_workers=4) as ex:
        f_cuda = ex.submit(build_cuda, verbose)
        f_diag = ex.submit(build_diag)
        f_oracle = ex.submit(build_oracle)
        f_ref = ex.submit(build_ref) if ref else None
        f_tobj = ex.submit(compile_torch_objects) if torch_layer else None
        out = {"cuda": f_cuda.result(), "diag": f_diag.result(), "oracle": f_oracle.result()}
        out["ref"] = f_ref.result() if f_ref else None
        if torch_layer:
            out["torch"] = build_torch(f_tobj.result())
    if ref and torch_layer:
        out["ref_caller"] = build_ref("caller")
    return out


if __name__ == "__main__":
    print(build_all(ref="--ref" in sys.argv, verbose="-v" in sys.argv))
