"""Build helper of the reference-shim check program (tests/gpu_kernels/shim_check.cpp)."""
import os
import shutil
import subprocess

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(REPO, "im-operator_gb300", "imop_gb300")
ORACLE = os.path.join(REPO, "oracle")


def cuda_libdir():
    for d in ("/usr/local/cuda/lib64", "/usr/local/cuda/targets/sbsa-linux/lib", "/usr/local/cuda/targets/x86_64-linux/lib"):
        if os.path.exists(os.path.join(d, "libcudart.so")):
            return d
    return "/usr/local/cuda/lib64"


def build_shim_check(out_path):
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-std=c++17", "-O1", os.path.join(REPO, "tests", "gpu_kernels", "shim_check.cpp"), "-o", out_path,
           "-I", os.path.join(REPO, "include"), "-L", LIBDIR, "-l:libimop_isp.so", "-L", ORACLE, "-l:liboracle_isp.so",
           "-L", cuda_libdir(), "-lcudart", f"-Wl,-rpath,{LIBDIR}:{ORACLE}:{cuda_libdir()}"]
    return subprocess.run(cmd, capture_output=True, text=True)
