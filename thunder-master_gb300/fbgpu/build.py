"""In-tree build of libfbgpu.so for sm_103a (GB300).

Translation units are compiled in parallel with nvcc and linked into
``fbgpu/_lib/libfbgpu.so``.  Host code is compiled with -ffp-contract=off so
the cutoff tests, grid indices and interpolation switches that must match the
reference exactly are never fused into FMAs by the host compiler (the GPU
box's aarch64 compiler would otherwise contract them).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(ROOT, "csrc")
OUT = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT, "libfbgpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                  "-Xcompiler", "-fPIC,-ffp-contract=off", "-Xptxas", "-v"]
SOURCES = ["fb_api.cu", "fb_fdata.cpp", "fb_neigh.cu", "fb_asm2c.cu", "fb_asm3c.cu", "fb_dasm2c.cu", "fb_dasm3c.cu",
           "fb_probe.cu", "fb_asm3c_df.cu", "fb_dasm3c_df.cu", "fb_mlp.cu", "fb_mlp_eval.cu", "fb_mlp_tc.cu", "fb_bloch.cu",
           "fb_pp.cu", "fb_ewald.cu", "fb_vxc.cu", "fb_vxc_df.cu", "fb_dogs_df.cu", "fb_solve.cu", "fb_ewald_df.cu"]
# Sources compiled in parts (-DFB_PART=k, k < count): their slow template
# instantiations compile in parallel (FB_IN_PART in fb_launch.h).
PARTS = {"fb_asm2c.cu": 4, "fb_asm3c.cu": 4, "fb_dasm2c.cu": 4, "fb_dasm3c.cu": 6, "fb_vxc.cu": 8}


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]


def _units():
    """(source, part or None) per compile job, slowest sources first."""
    units = []
    for s in _sources():
        n = PARTS.get(s)
        units += [(s, k) for k in range(n)] if n else [(s, None)]
    units.sort(key=lambda u: u[1] is None)
    return units


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(os.path.dirname(ROOT), "include", "fbgpu.h"))
    return files


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _deps() if os.path.exists(f))


def build(force=False, verbose=False):
    """Compile libfbgpu.so unless it is newer than every source."""
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()
    objs = []

    def compile_one(unit):
        src, part = unit
        stem = os.path.splitext(src)[0] + ("" if part is None else ".p%d" % part)
        obj = os.path.join(OUT, stem + ".o")
        extra = [] if part is None else ["-DFB_PART=%d" % part, "-diag-suppress=177"]
        cmd = [cc] + NVFLAGS + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
        return obj, r.stderr

    with ThreadPoolExecutor(max_workers=max(8, os.cpu_count() or 8)) as ex:
        results = list(ex.map(compile_one, _units()))
    logs = []
    for obj, log in results:
        objs.append(obj)
        logs.append(log)
    cmd = [cc] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + ["-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(LIB + ".tmp", LIB)
    with open(os.path.join(OUT, "ptxas.log"), "w") as f:
        f.write("\n".join(logs))
    if verbose:
        print("\n".join(logs))
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
