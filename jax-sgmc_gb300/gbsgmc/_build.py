"""Builds libgbsgmc.so from ``csrc/*.cu`` with nvcc for sm_103a.

The translation units are compiled in parallel into ``_build/`` and linked
with the static CUDA runtime into ``gbsgmc/_lib/libgbsgmc.so``.  A rebuild
happens only when a source or header is newer than the library.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
ROOT = PKG_DIR.parent
CSRC = ROOT / "csrc"
INCLUDE = ROOT.parent / "include"
BUILD_DIR = ROOT / "_build"
LIB_DIR = PKG_DIR / "_lib"
LIB_PATH = LIB_DIR / "libgbsgmc.so"

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-O2", "--expt-relaxed-constexpr"]


def nvcc_path() -> str:
  for cand in (os.environ.get("NVCC"), shutil.which("nvcc"),
               "/usr/local/cuda/bin/nvcc"):
    if cand and Path(cand).exists():
      return cand
  raise RuntimeError("nvcc not found: the gbsgmc CUDA library cannot be built")


def _sources():
  return sorted(CSRC.glob("*.cu"))


def _stale() -> bool:
  if not LIB_PATH.exists():
    return True
  t = LIB_PATH.stat().st_mtime
  deps = list(_sources()) + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h"))
  deps += list(INCLUDE.glob("*.h"))
  return any(p.stat().st_mtime > t for p in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
  """Compiles and links the library if needed; returns its path."""
  if not force and not _stale():
    return LIB_PATH
  nvcc = nvcc_path()
  BUILD_DIR.mkdir(exist_ok=True)
  LIB_DIR.mkdir(exist_ok=True)
  objs = []

  def compile_one(src: Path) -> Path:
    obj = BUILD_DIR / (src.stem + ".o")
    cmd = [nvcc, *ARCH_FLAGS, *NVCC_FLAGS, "-I", str(INCLUDE), "-c", str(src),
           "-o", str(obj)]
    if verbose:
      cmd.insert(1, "-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
      raise RuntimeError(f"nvcc failed on {src.name}:\n{res.stderr}")
    if verbose and res.stderr:
      print(res.stderr)
    return obj

  workers = min(len(_sources()), os.cpu_count() or 4)
  with cf.ThreadPoolExecutor(max_workers=workers) as ex:
    objs = list(ex.map(compile_one, _sources()))
  tmp = LIB_PATH.with_suffix(".so.tmp")
  cmd = [nvcc, *ARCH_FLAGS, "-shared", "-cudart", "static", "-o", str(tmp),
         *map(str, objs)]
  res = subprocess.run(cmd, capture_output=True, text=True)
  if res.returncode != 0:
    raise RuntimeError(f"nvcc link failed:\n{res.stderr}")
  os.replace(tmp, LIB_PATH)
  return LIB_PATH


if __name__ == "__main__":
  print(build(force=True, verbose=True))
