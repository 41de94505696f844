"""In-tree build of libtetemoko_gb300.so for sm_103a with nvcc.

Nine translation units, compiled in parallel:
  tmk_fp64.cu  plain FP64 kernels, --fmad=false (parity with the CPU oracle)
  tmk_fp32.cu  mixed-form kernels (FP32 volume, FP64 friction)
  tmk_capi.cu  the C ABI (host code)
  tmk_noalloc.cu  the allocation-free patch step (fixed device scratch array)
  tmk_amr.cu   coarse-fine coupling and the AMR hierarchy, --fmad=false
  tmk_regrid.cu  refinement tagging, --fmad=false
  tmk_3d.cu    the 3-D patch step (CH_SPACEDIM == 3), FP64 form, --fmad=false
  tmk_3d_f32.cu  its mixed form (FP32 volume arithmetic)
  tmk_level3d.cu  the 3-D device level (ghost exchange, batched step)
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libtetemoko_gb300.so")
BUILD = os.path.join(HERE, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
          "-Xcompiler", "-ffp-contract=off",   # host-computed launch constants: no FMA contraction
          "--expt-relaxed-constexpr", "-I", os.path.join(HERE, "..", "include")]
UNITS = {
    "tmk_fp64.cu": ["--fmad=false"],
    "tmk_fp32.cu": [],
    "tmk_capi.cu": [],
    "tmk_noalloc.cu": [],
    "tmk_amr.cu": ["--fmad=false"],
    "tmk_regrid.cu": ["--fmad=false"],
    "tmk_3d.cu": ["--fmad=false"],
    "tmk_3d_f32.cu": [],
    "tmk_level3d.cu": [],
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources_newer(target: str) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(HERE, "..", "include", "tetemoko_gb300.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    if not force and not _sources_newer(OUT):
        return OUT
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()

    def compile_unit(item):
        src, extra = item
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        cmd = [nv, *ARCH, *COMMON, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
        if ptxas_info:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        return obj, r.stdout + r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        results = list(ex.map(compile_unit, UNITS.items()))
    if verbose or ptxas_info:
        for _, log in results:
            if log.strip():
                print(log)
    tmp = OUT + ".tmp"
    cmd = [nv, *ARCH, "-shared", "-o", tmp, *[o for o, _ in results], "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    import sys
    print(build(force=True, verbose=True, ptxas_info="-v" in sys.argv))
