"""Build recipe for the reference's own CUDA near-field module (test and
measurement infrastructure only; nothing in the product imports this).

The reference ships its near-field correction as a torch C++/CUDA extension
(electrodrive/core/bem_near_cuda.cpp and bem_near_cuda_kernel.cu, loaded by
electrodrive/core/bem_near_cuda.py:93-123 through torch's JIT builder).  Its
pip install carries no C++/CUDA sources, so this recipe:

* ``copy_sources()`` (where the reference checkout exists) copies those two
  files, unmodified, into ``oracle/_ref/near_src/``;
* ``build()`` compiles them with nvcc and g++ against the installed torch's
  headers and libraries (the flags torch's extension builder uses, without
  its ninja dependency) into ``oracle/_ref/bem_near_cuda_ext*.so``, with the
  reference's own ``-O3 --use_fast_math`` and this GPU's architecture;
* ``load()`` imports it; its ``near_quadrature_matvec(V_far, sigma,
  centroids, areas, panel_vertices, near_pairs, K_E, quad_order)`` is the
  reference's native API (bem_near_cuda.cpp:239-271).

Everything it writes goes to ``oracle/_ref/`` (git-ignored).
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import importlib.util
import os
import shutil
import subprocess
import sys
import sysconfig
from typing import List, Optional

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
SRC_DIR = os.path.join(REF_DIR, "near_src")
NAME = "bem_near_cuda_ext"
SOURCES = ("bem_near_cuda.cpp", "bem_near_cuda_kernel.cu")
REL = "electrodrive/core"  # where the two files sit in the reference checkout


def reference_root() -> Optional[str]:
    root = os.environ.get("REFERENCE_ROOT") or "/root/reference"
    return root if os.path.isdir(os.path.join(root, REL)) else None


def copy_sources() -> bool:
    """Copy the reference's two source files into oracle/_ref/near_src (when
    the reference checkout is present); True if the sources are in place."""
    root = reference_root()
    if root is not None:
        os.makedirs(SRC_DIR, exist_ok=True)
        for f in SOURCES:
            src, dst = os.path.join(root, REL, f), os.path.join(SRC_DIR, f)
            if not os.path.exists(dst) or _digest(src) != _digest(dst):
                shutil.copyfile(src, dst)
    return all(os.path.exists(os.path.join(SRC_DIR, f)) for f in SOURCES)


def _digest(path: str) -> str:
    with open(path, "rb") as fh:
        return hashlib.sha256(fh.read()).hexdigest()


def lib_path() -> str:
    return os.path.join(REF_DIR, NAME + (sysconfig.get_config_var("EXT_SUFFIX") or ".so"))


def _torch_flags():
    import torch
    from torch.utils import cpp_extension as ce

    try:
        inc = ce.include_paths(device_type="cuda")
        libs = ce.library_paths(device_type="cuda")
    except TypeError:  # older keyword
        inc = ce.include_paths(cuda=True)
        libs = ce.library_paths(cuda=True)
    defs = [f"-DTORCH_EXTENSION_NAME={NAME}", "-DTORCH_API_INCLUDE_EXTENSION_H",
            f"-D_GLIBCXX_USE_CXX11_ABI={int(torch._C._GLIBCXX_USE_CXX11_ABI)}"]
    try:
        import warnings

        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            defs += list(ce._get_pybind11_abi_build_flags())
    except Exception:
        pass
    py_inc = sysconfig.get_paths()["include"]
    return inc + [py_inc], libs, defs


def build(force: bool = False) -> str:
    """Compile the copied reference sources; returns the module path."""
    if not copy_sources():
        raise RuntimeError("the reference near-field sources are not in oracle/_ref/near_src")
    out = lib_path()
    srcs = [os.path.join(SRC_DIR, f) for f in SOURCES]
    if not force and os.path.exists(out) and all(os.path.getmtime(out) > os.path.getmtime(s) for s in srcs):
        return out
    inc, libs, defs = _torch_flags()
    I = [f"-I{p}" for p in inc]
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(nvcc)), "include")
    objs = [os.path.join(REF_DIR, f + ".o") for f in SOURCES]
    cmds: List[List[str]] = [
        ["g++", "-c", srcs[0], "-o", objs[0], "-O3", "-std=c++17", "-fPIC", f"-I{cuda_inc}", *I, *defs],
        [nvcc, "-c", srcs[1], "-o", objs[1], "-O3", "--use_fast_math", "-std=c++17",
         "-gencode", "arch=compute_103a,code=sm_103a", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-D__CUDA_NO_HALF_OPERATORS__", "-D__CUDA_NO_HALF_CONVERSIONS__", "-D__CUDA_NO_BFLOAT16_CONVERSIONS__",
         "-D__CUDA_NO_HALF2_OPERATORS__", *I, *defs],
    ]
    with cf.ThreadPoolExecutor(2) as ex:
        for cmd, r in zip(cmds, ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), cmds)):
            if r.returncode != 0:
                raise RuntimeError("compile failed: " + " ".join(cmd[:3]) + "\n" + r.stderr[-3000:])
    L = [f"-L{p}" for p in libs]
    rpath = [f"-Wl,-rpath,{p}" for p in libs]
    link = ["g++", "-shared", *objs, "-o", out, *L, *rpath, "-lc10", "-ltorch", "-ltorch_cpu", "-ltorch_python",
            "-lc10_cuda", "-ltorch_cuda", f"-L{os.path.join(os.path.dirname(os.path.dirname(nvcc)), 'lib64')}",
            "-lcudart"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stderr[-3000:])
    return out


def load():
    """The compiled reference module (builds it first if needed)."""
    import torch  # noqa: F401  (the module links against torch's libraries)

    path = build()
    spec = importlib.util.spec_from_file_location(NAME, path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


if __name__ == "__main__":
    print(build(force="-f" in sys.argv))
