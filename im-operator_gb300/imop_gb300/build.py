"""Build recipe of the CUDA library (sm_103a) and the CPU oracle.

    python -m imop_gb300.build            # from im-operator_gb300/, or via __graft_entry__.build()

Every translation unit under csrc/ is compiled by nvcc in parallel into _build/, then linked
into imop_gb300/libimop_isp.so.  Host code is compiled with -ffp-contract=off so that host-side
parameter derivations (polynomial shading radius, flat-field grid) round exactly like the
reference's CPU code; device arithmetic on the parity path uses explicit rounding intrinsics.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)                 # im-operator_gb300/
REPO = os.path.dirname(ROOT)
CSRC = os.path.join(ROOT, "csrc")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "libimop_isp.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fPIC,-ffp-contract=off,-fopenmp,-O3",
              "-I", os.path.join(REPO, "include")]


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    out = []
    for f in sorted(os.listdir(CSRC)):
        if f.endswith(".cu") or f.endswith(".cpp"):
            out.append(os.path.join(CSRC, f))
    return out


def _deps_newer(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    hdrs = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh", ".inl"))]
    hdrs.append(os.path.join(REPO, "include", "imop_isp.h"))
    return any(os.path.getmtime(p) > t for p in [src] + hdrs)


def _compile(src, verbose):
    nvcc = _nvcc()
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if not _deps_newer(obj, src):
        return obj
    cmd = [nvcc] + ARCH + NVCC_FLAGS + ["-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build_library(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if os.path.exists(LIB) and all(os.path.getmtime(o) <= os.path.getmtime(LIB) for o in objs):
        return LIB
    cmd = [_nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-Xcompiler", "-fopenmp", "-lcudart"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


def build_oracle(verbose=False):
    """The CPU oracle (test infrastructure), and the reference's own CPU library (its dispatchers
    over this library, and its own GPU glue for the timed reference arm) where the reference's
    sources exist: the reference tree
    (IMOP_REFERENCE_ROOT, default the checkout beside this one) is first copied into the
    git-ignored oracle/_ref/src, so a host without the tree builds the same files from the copy."""
    oracle = os.path.join(REPO, "oracle")
    r = subprocess.run(["make", "-C", oracle, "-j8"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    ref_root = os.environ.get("IMOP_REFERENCE_ROOT", "/root/reference")
    if os.path.isdir(os.path.join(ref_root, "src", "algorithms")):
        r = subprocess.run(["make", "-C", oracle, "stage", f"REF_ROOT={ref_root}"], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"staging the reference sources failed:\n{r.stdout}\n{r.stderr}")
    staged = os.path.join(oracle, "_ref", "src")
    if os.path.isdir(os.path.join(staged, "src", "algorithms")):
        jobs = str(min(16, os.cpu_count() or 4))
        r = subprocess.run(["make", "-C", oracle, "ref", "dropin", "refcuda", "-j" + jobs, f"REF_ROOT={staged}"],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference build failed:\n{r.stdout}\n{r.stderr}")


def build_all(verbose=False):
    build_library(verbose)
    build_oracle(verbose)


if __name__ == "__main__":
    build_all(verbose="-v" in sys.argv)
