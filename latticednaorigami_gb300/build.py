"""Compiles the engine's CUDA kernels and C++ host library into an in-tree
shared library (libldo_gb300.so) for sm_103a.  No CMake: the compiler
invocations run in parallel, then one link."""
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libldo_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path():
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; the engine needs the CUDA toolkit to build")
    return cand


def cuda_include():
    nvcc = nvcc_path()
    root = os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return os.path.join(root, "include")


def _run_all(cmds):
    procs = [subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True) for c in cmds]
    for c, p in zip(cmds, procs):
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("build step failed: %s\n%s" % (" ".join(c), out))


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    nvcc = nvcc_path()
    k_obj = os.path.join(BUILD, "ldo_kernels.o")
    m_obj = os.path.join(BUILD, "ldo_mlp.o")
    e_obj = os.path.join(BUILD, "ldo_enum.o")
    h_obj = os.path.join(BUILD, "ldo_host.o")
    cmds = [
        [nvcc] + ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-c", os.path.join(CSRC, "ldo_kernels.cu"), "-o", k_obj],
        [nvcc] + ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-c", os.path.join(CSRC, "ldo_mlp.cu"), "-o", m_obj],
        [nvcc] + ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-c", os.path.join(CSRC, "ldo_enum.cu"), "-o", e_obj],
        ["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-I" + cuda_include(),
         "-c", os.path.join(CSRC, "ldo_host.cpp"), "-o", h_obj],
    ]
    _run_all(cmds)
    tmp = LIB + ".tmp"
    _run_all([[nvcc] + ARCH + ["-shared", "-Xcompiler", "-fPIC", k_obj, m_obj, e_obj, h_obj, "-o", tmp]])
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
