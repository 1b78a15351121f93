"""Build ``libgbxtb.so`` (the CUDA engine and its C ABI) in-tree for sm_103a,
and the torch operators over it.

``python -m dxtb_gb300.build`` compiles every ``csrc/*.cu`` translation unit
in parallel with nvcc and links them into ``dxtb_gb300/libgbxtb.so``; then
``csrc/torch_ops.cpp`` (``TORCH_LIBRARY(gbxtb, m)``: ``torch.ops.gbxtb.*``)
is compiled against torch and that library into
``dxtb_gb300/_build/torch_ops/gbxtb_torch_ops.so``.  Objects go to
``dxtb_gb300/_build/`` (git-ignored).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libgbxtb.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
    "-Xcompiler", "-Wall", "-I", str(PKG.parent / "include")]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgbxtb.so")


TORCH_OPS_SRC = CSRC / "torch_ops.cpp"
TORCH_OPS_DIR = BUILD / "torch_ops"
TORCH_OPS_NAME = "gbxtb_torch_ops"


def torch_ops_path() -> Path:
    return TORCH_OPS_DIR / f"{TORCH_OPS_NAME}.so"


def build_torch_ops(verbose: bool = False) -> Path:
    """Compile and load the torch operators (needs libgbxtb.so built)."""
    from torch.utils import cpp_extension

    out = torch_ops_path()
    deps = [TORCH_OPS_SRC, PKG.parent / "include" / "gbxtb.h", LIB]
    if out.exists() and any(d.exists() and d.stat().st_mtime > out.stat().st_mtime for d in deps):
        shutil.rmtree(TORCH_OPS_DIR)  # the C ABI changed: rebuild from scratch
    TORCH_OPS_DIR.mkdir(parents=True, exist_ok=True)
    cuda_home = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
    cpp_extension.load(
        name=TORCH_OPS_NAME,
        sources=[str(TORCH_OPS_SRC)],
        extra_cflags=["-O2"],
        extra_include_paths=[str(PKG.parent / "include"), str(cuda_home / "include")],
        extra_ldflags=[f"-L{PKG}", "-lgbxtb", f"-Wl,-rpath,{PKG}"],
        build_directory=str(TORCH_OPS_DIR),
        with_cuda=True,
        is_python_module=False,
        verbose=verbose,
    )
    return torch_ops_path()


def _sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = list(CSRC.glob("*")) + [PKG.parent / "include" / "gbxtb.h", Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps if p.exists())


def build(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None) -> Path:
    if not force and not _stale():
        return LIB
    BUILD.mkdir(exist_ok=True)
    cc = nvcc()
    flags = NVCC_FLAGS + (extra_flags or [])

    def compile_one(src: Path) -> Path:
        obj = BUILD / (src.stem + ".o")
        cmd = [cc, *ARCH, *flags, "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr, file=sys.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        objs = list(ex.map(compile_one, _sources()))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc, *ARCH, "-shared", "-Xlinker", "-soname=libgbxtb.so", "-o", str(tmp), *map(str, objs)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    tmp.replace(LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
    if "--no-torch-ops" not in sys.argv:
        print(build_torch_ops(verbose="-v" in sys.argv))
