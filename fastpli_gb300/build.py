"""Builds libfastpli_gb300.so (sm_103a) in-tree with nvcc.

Each translation unit is compiled in parallel, then linked into
``fastpli_gb300/_lib/libfastpli_gb300.so``.  No cmake, no torch extension
machinery: the library exposes a plain C ABI (``include/fastpli_gb300.h``).

Flags that matter for parity:
  * host code: ``-ffp-contract=off`` — the host planning replays the
    reference's double arithmetic (segment boxes, ray geometry) and must not
    fuse multiply-adds (GCC fuses by default on aarch64).
  * ``tissue.cu``, ``voxel_bricks.cu``: ``-fmad=false`` — the voxelizer's
    exact double path must round every product and sum separately, as the
    reference does.
  * ``raymarch.cu``, ``batch.cu``: ``-fmad=false`` with the wanted fused
    multiply-adds written out — every march kernel (plain or batched,
    per-thread or cooperative) then gives the same bits for the same tile.
  * ``optic.cu``: ``-fmad=false`` — the Gaussian filter sums in scipy's
    order with separate roundings.
  * ``rofl.cu``: ``-fmad=false`` — MINPACK's and numpy's sums and products
    round separately; the fused forms numpy's matrix product uses are
    written out.
"""

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(HERE, "_lib", "obj")
LIB_NAME = "libfastpli_gb300.so"
LIB_PATH = os.path.join(OUT_DIR, LIB_NAME)
# throughput microbenchmarks for the roofline (bench.py), outside the path's ABI
PEAKS_SRC = os.path.join(CSRC, "peaks", "peaks.cu")
PEAKS_LIB = os.path.join(OUT_DIR, "libfpgb_peaks.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
          "-I", os.path.join(ROOT, "include")]
PER_FILE = {"capi.cu": ["-Xcompiler", "-fopenmp"],
            "tissue.cu": ["-fmad=false", "-Xcompiler", "-fopenmp"],
            "voxel_bricks.cu": ["-fmad=false"],
            "optic.cu": ["-fmad=false"],
            "rofl.cu": ["-fmad=false"],
            "raymarch.cu": ["-fmad=false"],
            "batch.cu": ["-fmad=false", "-Xcompiler", "-fopenmp"]}


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _compile(nvcc, src, extra):
    obj = os.path.join(OBJ_DIR, src.replace(".cu", ".o"))
    cmd = [nvcc, *ARCH, *COMMON, *PER_FILE.get(src, []), *extra, "-c",
           os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def _stale():
    if not os.path.exists(LIB_PATH) or not os.path.exists(PEAKS_LIB):
        return True
    t = os.path.getmtime(LIB_PATH)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [PEAKS_SRC]
    deps += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    deps.append(__file__)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, extra=()):
    """Compile and link the library if any source is newer.  Returns the path."""
    if not force and not _stale():
        return LIB_PATH
    nvcc = _nvcc()
    os.makedirs(OBJ_DIR, exist_ok=True)
    extra = list(extra)
    def peaks():
        r = subprocess.run([nvcc, *ARCH, *COMMON, "-shared", PEAKS_SRC, "-o", PEAKS_LIB],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on peaks.cu:\n{r.stdout}\n{r.stderr}")

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        peaks_job = ex.submit(peaks)
        results = list(ex.map(lambda s: _compile(nvcc, s, extra), sources()))
        peaks_job.result()
    objs = [o for o, _ in results]
    if verbose:
        for _, err in results:
            if err.strip():
                print(err, file=sys.stderr)
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart", "-lgomp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True,
                extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else []))
