"""In-tree build of the CUDA library libati.so for sm_103a.

Every translation unit is compiled by nvcc in parallel (one -gencode, no
cmake), then linked into tandemproject_gb300/_build/libati.so.  Rebuilds only
when a source is newer than the library.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libati.so")
ROOT = os.path.dirname(HERE)
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code: no FMA contraction (gcc contracts by default on aarch64), so the
# scheme coefficients are identical on x86 and Arm
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off", "--expt-relaxed-constexpr"]
# (source, object, extra flags): the kernels are compiled twice, with and
# without FMA contraction; set-up kernels never contract
SOURCES = [
    ("ati_kernels.cu", "ati_kernels_fast.o", ["-DATI_KNS=fast", "-DATI_KFAST=1", "-fmad=true"]),
    ("ati_kernels.cu", "ati_kernels_strict.o", ["-DATI_KNS=strict", "-DATI_KFAST=0", "-fmad=false"]),
    ("ati_api.cu", "ati_api.o", ["-fmad=false"]),
    ("ati_scheme.cpp", "ati_scheme.o", []),
    ("ati_probe.cu", "ati_probe.o", []),
    ("ati_noalloc.cu", "ati_noalloc.o", ["-fmad=false"]),
    ("ati_io.cpp", "ati_io.o", []),
    ("ati_turb.cu", "ati_turb.o", []),
    ("ati_convert.cu", "ati_convert.o", []),
]


def _deps():
    out = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    out.append(os.path.join(ROOT, "include", "ati.h"))
    return out


def build(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in _deps()):
            return LIB
    nvcc = NVCC if os.path.exists(NVCC) else "nvcc"

    def compile_one(item):
        src, objname, extra = item
        obj = os.path.join(OUT, objname)
        cmd = [nvcc, *ARCH, *FLAGS, *extra, "-x", "cu", "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
