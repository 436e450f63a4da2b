"""Build recipe for libmocatgb.so (in-tree, sm_103a only).

Each translation unit is compiled by nvcc in parallel, then linked into
``mocat_gb300/_build/libmocatgb.so`` against the shared CUDA runtime, so a
process that already loaded PyTorch's libcudart.so.13 shares that runtime.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libmocatgb.so")

SOURCES = ["mgb_rng.cu", "mgb_resample.cu", "mgb_pf_lg.cu", "mgb_pf_persist.cu", "mgb_noalloc.cu", "mgb_pf_sv_batch.cu", "mgb_pf_opt.cu", "mgb_pf_adjoint.cu", "mgb_pf_score.cu", "mgb_smc.cu", "mgb_logreg_tc.cu", "mgb_ffbsi.cu", "mgb_rejection.cu", "mgb_pf_nl1d.cu", "mgb_pf_sv.cu", "mgb_abc.cu", "mgb_kalman.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fno-strict-aliasing",
                     "-Xptxas", "-warn-spills"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: libmocatgb.so cannot be built")


def _stale(obj, src):
    if not os.path.exists(obj):
        return True
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    deps.append(os.path.join(HERE, "..", "include", "mocat_gb300.h"))
    return any(os.path.getmtime(d) > os.path.getmtime(obj) for d in deps if os.path.exists(d))


def build(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        if force or _stale(o, s):
            jobs.append([cc] + NVCC_FLAGS + ["-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(run, jobs))
    objs = [os.path.join(BUILD, s.replace(".cu", ".o")) for s in SOURCES]
    if jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        run([cc] + ARCH + ["-shared", "-cudart", "shared", "-o", tmp] + objs +
            ["-Xlinker", "-rpath=/usr/local/cuda/lib64"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
