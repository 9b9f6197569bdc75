"""In-tree build of libsffg.so: nvcc for the sm_103a kernels, g++ for the
host code, linked into one shared library under nabc_gb300/_lib/.

Objects are rebuilt when their source or any local header is newer.  The
translation units compile in parallel so a clean build takes about a
minute.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
# SFFG_BUILD_DIR and SFFG_NVCC_EXTRA build a variant (e.g. another tuning
# constant, -DSFFG_GROUP=8) into another directory; load it with
# SFFG_LIBRARY=<dir>/libsffg.so.
OUT = os.environ.get("SFFG_BUILD_DIR", os.path.join(PKG, "_lib"))
ROOT = os.path.dirname(PKG)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas", "-O3",
              "--expt-relaxed-constexpr"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-Wno-unused-function"]
# Host files whose arithmetic must match the reference's bit for bit on any
# host: no floating-point contraction (FMA) and the C++20 coroutines the
# minimiser and the low-mode search are written with.
CXX_FILE_FLAGS = {
    "xmin.cpp": ["-std=c++20", "-ffp-contract=off"],
    "lmod.cpp": ["-std=c++20", "-ffp-contract=off"],
    "lowmodes.cpp": ["-ffp-contract=off"],
    # the synthetic-molecule generator: the same molecules on every host, and
    # the same bits as its C restatement under oracle/ (which the CPU
    # baseline generates its inputs with)
    "synth.cpp": ["-ffp-contract=off"],
}


def library_path():
    return os.environ.get("SFFG_LIBRARY", os.path.join(OUT, "libsffg.so"))


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libsffg")


def _newest_header():
    hs = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h"))
    return max(os.path.getmtime(h) for h in hs)


def _compile(src, obj, force):
    if not force and os.path.exists(obj) and \
            os.path.getmtime(obj) >= max(os.path.getmtime(src), _newest_header()):
        return None
    if src.endswith(".cu"):
        cmd = [_nvcc()] + ARCH + NVCC_FLAGS + os.environ.get("SFFG_NVCC_EXTRA", "").split() + \
            ["-I", CSRC, "-c", src, "-o", obj]
    else:
        cmd = ["g++"] + CXX_FLAGS + CXX_FILE_FLAGS.get(os.path.basename(src), []) + ["-I", CSRC, "-I", "/usr/local/cuda/include", "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stderr


def build(force=False, verbose=False, report=False):
    """Compile every translation unit and link libsffg.so; returns its path.
    report: print which translation units were compiled (the others were up
    to date), for which architecture, and where the library is."""
    os.makedirs(OUT, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    objs = [os.path.join(OUT, os.path.basename(s) + ".o") for s in srcs]
    compiled = []
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        futs = [ex.submit(_compile, s, o, force) for s, o in zip(srcs, objs)]
        for s, f in zip(srcs, futs):
            msg = f.result()
            if msg is not None:
                compiled.append(os.path.basename(s))
            if verbose and msg:
                print(msg)
    lib = os.path.join(OUT, "libsffg.so")
    if force or not os.path.exists(lib) or os.path.getmtime(lib) < max(os.path.getmtime(o) for o in objs):
        cmd = [_nvcc()] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if report:
            print(f"libsffg: linked {lib}")
    if report:
        print(f"libsffg: compiled {len(compiled)} of {len(srcs)} translation units for {ARCH[1]}"
              f"{': ' + ', '.join(compiled) if compiled else ' (all up to date)'}")
    return lib


if __name__ == "__main__":
    print(build(verbose=True))
