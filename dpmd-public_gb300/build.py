"""Build libgbdp.so (the C-ABI CUDA library) in-tree for sm_103a, and
libdeepmd_op_gb300.so (the libtorch registration of the deepmd operators
over it, for C++ TorchScript hosts).

Each CUDA translation unit under csrc/ is compiled to an object in parallel
(the libtorch shim alongside), then linked beside this file.  Rebuilds only
what a newer source or header affects.
"""

from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgbdp.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "-Xcompiler",
    "-fPIC,-ffp-contract=off,-fvisibility=hidden",
    "-I" + os.path.join(ROOT, "include"),
]


TORCH_SRC = os.path.join(CSRC, "torch_ops.cpp")
TORCH_LIB = os.path.join(HERE, "libdeepmd_op_gb300.so")


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgbdp.so")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps():
    return _sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(
        os.path.join(ROOT, "include", "*.h"))


def needs_build() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in _deps()) or os.path.getmtime(__file__) > t


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(OBJ, os.path.basename(src)[:-3] + ".o")
    cmd = [nvcc()] + NVCC_FLAGS + extra + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stderr}")
    return obj


def _torch_flags():
    import torch
    import torch.utils.cpp_extension as ce

    inc = [f"-I{p}" for p in ce.include_paths()]
    lib = ce.library_paths()[0]
    abi = int(torch._C._GLIBCXX_USE_CXX11_ABI)
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(nvcc())), "include")
    return (["-O2", "-std=c++17", "-fPIC", f"-D_GLIBCXX_USE_CXX11_ABI={abi}",
             "-I" + os.path.join(ROOT, "include"), "-I" + cuda_inc] + inc,
            [f"-L{lib}", f"-Wl,-rpath,{lib}", "-ltorch", "-ltorch_cpu", "-lc10", "-lc10_cuda"])


def _compile_torch_shim() -> str:
    """The libtorch registration of the deepmd operators (a C++ TorchScript
    host loads it in place of the reference's libdeepmd_op_pt.so)."""
    cxx = shutil.which("g++") or "g++"
    cflags, _ = _torch_flags()
    obj = os.path.join(OBJ, "torch_ops.o")
    r = subprocess.run([cxx] + cflags + ["-c", TORCH_SRC, "-o", obj], capture_output=True,
                       text=True)
    if r.returncode != 0:
        raise RuntimeError(f"g++ failed on torch_ops.cpp:\n{r.stderr[-4000:]}")
    return obj


def _torch_needs_build() -> bool:
    if not os.path.exists(TORCH_LIB):
        return True
    t = os.path.getmtime(TORCH_LIB)
    deps = [TORCH_SRC, __file__] + glob.glob(os.path.join(ROOT, "include", "*.h"))
    return any(os.path.getmtime(p) > t for p in deps)


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    if not force and not needs_build() and not _torch_needs_build():
        return LIB
    os.makedirs(OBJ, exist_ok=True)
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        shim = ex.submit(_compile_torch_shim) if (force or _torch_needs_build()) else None
        if force or needs_build():
            objs = list(ex.map(lambda s: _compile(s, extra), _sources()))
            tmp = LIB + ".tmp"
            cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcublas"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"link failed:\n{r.stderr}")
            os.replace(tmp, LIB)
        shim_obj = shim.result() if shim else None
    if shim_obj:
        _, ldflags = _torch_flags()
        tmp = TORCH_LIB + ".tmp"
        cmd = [shutil.which("g++") or "g++", "-shared", "-o", tmp, shim_obj, "-L" + HERE,
               "-Wl,-rpath,$ORIGIN", "-lgbdp"] + ldflags
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link of libdeepmd_op_gb300.so failed:\n{r.stderr[-4000:]}")
        os.replace(tmp, TORCH_LIB)
    return LIB


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
