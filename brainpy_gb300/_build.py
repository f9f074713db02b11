"""Build recipe for libbpgpu.so (the CUDA kernels and their C ABI).

Every ``.cu`` file under ``csrc/`` is compiled for sm_103a in parallel and linked
into ``brainpy_gb300/libbpgpu.so``, in tree.  nvcc cross-compiles, so this runs
without a GPU.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libbpgpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xptxas", "-warn-spills"]


def nvcc():
  exe = shutil.which("nvcc")
  if exe is None:
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
      return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libbpgpu.so")
  return exe


def _newer(target, sources):
  if not os.path.exists(target):
    return True
  t = os.path.getmtime(target)
  return any(os.path.getmtime(s) > t for s in sources)


def build_library(force=False, verbose=False, extra_flags=()):
  os.makedirs(BUILD, exist_ok=True)
  sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
  headers = sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
                   + glob.glob(os.path.join(PKG, "..", "include", "*.h")))
  objs = []
  jobs = []
  for src in sources:
    obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
    objs.append(obj)
    if force or _newer(obj, [src] + headers):
      cmd = [nvcc()] + ARCH + NVCC_FLAGS + list(extra_flags) + ["-c", src, "-o", obj]
      jobs.append(cmd)
  if jobs:
    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
      results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
    for cmd, r in zip(jobs, results):
      if verbose or r.returncode != 0:
        print(" ".join(cmd))
        print(r.stdout + r.stderr)
      if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {cmd[-3]}")
  if force or jobs or _newer(LIB, objs):
    cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
      print(" ".join(cmd))
      print(r.stdout + r.stderr)
      raise RuntimeError("linking libbpgpu.so failed")
  return LIB


if __name__ == "__main__":
  print(build_library(verbose=True))
