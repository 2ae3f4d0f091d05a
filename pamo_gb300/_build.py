"""In-tree build of the CUDA library ``pamo_gb300/_lib/libpamo_gb300.so`` for sm_103a, and of the PyTorch extension
module ``pamo_gb300._C`` that binds it under the reference's operator names.

Each translation unit is compiled by nvcc in parallel with ``--fmad=false`` (the reference's float semantics:
no contraction of multiply-add) and host code with ``-ffp-contract=off``, then linked into one shared
library that exports the C ABI of include/pamo_gb300.h.
"""

from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
LIBNAME = "libpamo_gb300.so"
SOURCES = ["scan.cu", "lbvh.cu", "simp_round.cu", "pamo_ctx.cu", "noalloc.cu", "safe_project.cu", "batch.cu",
           "batch_round.cu", "metrics.cu", "remesh.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "--fmad=false", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2"]


def nvcc_path() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build pamo_gb300")


def lib_path() -> str:
    return os.path.join(LIBDIR, LIBNAME)


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def torch_ext_path() -> str:
    """Path of the PyTorch extension module pamo_gb300._C (the reference's operator module pamo._C)."""
    import sysconfig

    return os.path.join(HERE, "_C" + sysconfig.get_config_var("EXT_SUFFIX"))


TORCH_EXT_OBJ = os.path.join(LIBDIR, "obj", "torch_ext.o")


def _torch_ext_cmd():
    """g++ compile and link commands of the extension module: torch headers for the tensor plumbing, linked to libpamo_gb300.so (found
    next to it through the rpath) for all compute."""
    import sysconfig

    import torch
    import torch.utils.cpp_extension as ce

    try:
        incs, libs = ce.include_paths("cuda"), ce.library_paths("cuda")
    except TypeError:  # older signature: include_paths(cuda=True)
        incs, libs = ce.include_paths(cuda=True), ce.library_paths(cuda=True)
    abi = int(bool(torch._C._GLIBCXX_USE_CXX11_ABI))
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-DTORCH_EXTENSION_NAME=_C", "-DTORCH_API_INCLUDE_EXTENSION_H",
           f"-D_GLIBCXX_USE_CXX11_ABI={abi}", f"-I{sysconfig.get_paths()['include']}"]
    compile_cmd = cmd + [f"-I{d}" for d in incs] + ["-c", os.path.join(CSRC, "torch_ext.cpp"), "-o", TORCH_EXT_OBJ]
    link_cmd = ["g++", "-shared", "-fPIC", TORCH_EXT_OBJ, "-o", torch_ext_path()]
    link_cmd += [f"-L{d}" for d in libs] + [f"-Wl,-rpath,{d}" for d in libs]
    link_cmd += ["-lc10", "-lc10_cuda", "-ltorch", "-ltorch_cpu", "-ltorch_python", "-lcudart", f"-L{LIBDIR}",
                 "-lpamo_gb300", "-Wl,-rpath,$ORIGIN/_lib"]
    return compile_cmd, link_cmd


def build(force: bool = False, verbose: bool = False, torch_ext: bool = True) -> str:
    """Compile the library (and, with torch_ext, the extension module pamo_gb300._C) if a source is newer than
    it; returns the library's path."""
    os.makedirs(os.path.join(LIBDIR, "obj"), exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "pamo_gb300.h"))
    nvcc = nvcc_path()
    objs = []
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(LIBDIR, "obj", src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc, *ARCH, *NVCC_FLAGS, "-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)

    ext_link = None
    if torch_ext:  # compiled beside the CUDA units, linked once the library exists
        ext_cc, ext_link = _torch_ext_cmd()
        ext_deps = [os.path.join(CSRC, "torch_ext.cpp"), os.path.join(os.path.dirname(HERE), "include", "pamo_gb300.h")]
        if force or _stale(TORCH_EXT_OBJ, ext_deps):
            jobs.append(ext_cc)
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(run, jobs))
    out = lib_path()
    if force or jobs or _stale(out, objs):
        run([nvcc, "-shared", *ARCH, "-o", out, *objs, "-lcudart", "-Xcompiler", "-pthread"])
    if ext_link and (force or _stale(torch_ext_path(), [TORCH_EXT_OBJ, out])):
        run(ext_link)
    return out


if __name__ == "__main__":
    print(build(verbose=True))
