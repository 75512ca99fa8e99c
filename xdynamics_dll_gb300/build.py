"""Builds libxdem_gb300.so in-tree for sm_103a.

Each .cu unit compiles in parallel with nvcc; the FP64 units use -fmad=false
so their arithmetic rounds operation by operation like the CPU oracle.  The
mixed form's sphere unit uses -fmad=false too: its FMAs are the explicit fmaf
of the float-pair helpers, so a contact computes the same bits whether the
walk, the candidate list or a separately compiled call evaluates it
(implicit contraction depends on the inlining context).  Its mesh and
cluster-body unit contracts: FP64 geometry there runs on the slow FP64 pipe.
Host code is compiled without
contraction too (-ffp-contract=off), so host-side setup math is identical on
x86 and Arm.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libxdem_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                 "-Xcompiler", "-fvisibility=hidden",
                 "-diag-suppress", "1444", "-Xptxas", "-warn-spills"]
UNITS = {
    "xdem_kernels.cu": ["-fmad=false"],
    "xdem_sort.cu": [],
    "xdem_api.cu": ["-fmad=false"],
    "xdem_sim.cu": ["-fmad=false"],
    "xdem_fused_host.cu": ["-fmad=false"],
    "xdem_fused_fp64.cu": ["-fmad=false"],
    "xdem_fused_mixed.cu": ["-fmad=false"],
    "xdem_fused_mixed_mesh.cu": ["-fmad=true"],
    "xdem_noalloc.cu": [],
    "xdem_adjoint.cu": ["-fmad=false"],
    "xdem_tune.cu": [],
    "xdem_io.cu": [],
    "xdem_hht.cu": ["-fmad=false"],
}


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _compile(unit, flags, verbose):
    src = os.path.join(CSRC, unit)
    obj = os.path.join(BUILD, unit.replace(".cu", ".o"))
    cmd = [nvcc()] + COMMON + flags + (["-Xptxas", "-v"] if verbose else []) + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {unit}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(os.path.dirname(HERE), "include", "xdem_c.h"))
    deps.append(os.path.abspath(__file__))
    return all(os.path.getmtime(d) <= t for d in deps)


def build(force=False, verbose=False):
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(len(UNITS), os.cpu_count() or 4)) as ex:
        futs = {ex.submit(_compile, u, f, verbose): u for u, f in UNITS.items()}
        objs = []
        for fu in cf.as_completed(futs):
            obj, log = fu.result()
            objs.append(obj)
            if verbose and log:
                sys.stderr.write(f"--- {futs[fu]}\n{log}")
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + sorted(objs)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
