"""Build the cosmos_gb300 CUDA library in-tree for sm_103a.

    python -m cosmos_gb300.build [--verbose] [--ptxas-v]

Produces cosmos_gb300/libcosmos_gb300.so from cosmos_gb300/csrc/*.cu.  The translation unit
holding the reference-exact FP64 kernels is compiled with --fmad=false (no contraction of
a*b+c into FMA, which the reference's x86/Arm builds do not do either); the FP32 unit keeps FMA.
Objects are compiled in parallel; nothing is rebuilt when sources are unchanged.
"""
import argparse
import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libcosmos_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr", "-I", CSRC,
          "-I", INCLUDE]
# per-unit extra flags
UNITS = {
    "kernels_exact.cu": ["--fmad=false"],
    "kernels_fast.cu": [],
    "kernels_sr_fast.cu": [],
    "kernels_gr_fast.cu": [],
    "kernels_batch_fast.cu": [],
    "kernels_batch_exact.cu": ["--fmad=false"],
    "kernels_adjoint.cu": ["--fmad=false"],
    "kernels_adjoint_fast.cu": [],
    "kernels_adjoint_rel.cu": ["--fmad=false"],
    "capi.cu": [],
    "capi_batch.cu": [],
    "noalloc.cu": [],
    "capi_adjoint.cu": [],
    "capi_amr.cu": [],
    "capi_state.cu": [],
}


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _digest(paths, flags):
    h = hashlib.sha256()
    for p in sorted(paths):
        with open(p, "rb") as f:
            h.update(f.read())
    h.update(" ".join(flags).encode())
    return h.hexdigest()


def _headers():
    out = []
    for d in (CSRC, INCLUDE):
        for n in os.listdir(d):
            if n.endswith((".cuh", ".h", ".hpp")):
                out.append(os.path.join(d, n))
    return out


def build(verbose=False, ptxas_v=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    hdrs = _headers()
    units = [u for u in UNITS if os.path.exists(os.path.join(CSRC, u))]
    jobs = []
    for u in units:
        src = os.path.join(CSRC, u)
        obj = os.path.join(BUILD, u.replace(".cu", ".o"))
        flags = ARCH + COMMON + UNITS[u] + (["-Xptxas", "-v"] if ptxas_v else [])
        stamp = obj + ".sha"
        dig = _digest([src] + hdrs, flags)
        if not force and os.path.exists(obj) and os.path.exists(stamp) and open(stamp).read() == dig:
            continue
        jobs.append((u, [cc, "-c", src, "-o", obj] + flags, stamp, dig))
    def run(job):
        name, cmd, stamp, dig = job
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {name}:\n{r.stdout}\n{r.stderr}")
        if ptxas_v or verbose:
            sys.stderr.write(r.stderr)
        with open(stamp, "w") as f:
            f.write(dig)
        return name
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for _ in ex.map(run, jobs):
                pass
    objs = [os.path.join(BUILD, u.replace(".cu", ".o")) for u in units]
    if jobs or not os.path.exists(LIB):
        cmd = [cc, "-shared", "-o", LIB] + objs + ARCH + ["-Xcompiler", "-fPIC", "-lcuda"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--verbose", action="store_true")
    ap.add_argument("--ptxas-v", action="store_true")
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args()
    print(build(verbose=a.verbose, ptxas_v=a.ptxas_v, force=a.force))


if __name__ == "__main__":
    main()
