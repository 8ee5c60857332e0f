"""Build recipe for the GB300 SGM engine (no cmake; nvcc + gcc only).

Outputs, all under sgm-bench_gb300/_build/ (git-ignored):
  libsgmgb.so                    the engine and its C ABI (include/sgmgb.h)
  libsgm_gb300_d{D}_p{P}.so      the sgm.h plugin (SGM_IMPL) for one compile-time D/paths
  sgmgb_cli                      command-line front end (sgm_ms-style and harness-style runs)
Every CUDA translation unit is compiled for sm_103a only.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc")
CC = os.environ.get("CC", "gcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "-I" + os.path.join(ROOT, "include")]
CFLAGS = ["-O2", "-fPIC", "-std=gnu11", "-Wall", "-Wextra", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include")]

CU_SOURCES = ["sgmgb_kernels.cu", "sgmgb_path.cu", "sgmgb_runtime.cu", "sgmgb_batch.cu", "sgmgb_server.cu",
              "sgmgb_noalloc.cu", "sgmgb_sum.cu", "sgmgb_fused.cu", "sgmgb_post.cu"]
C_SOURCES = ["synth.c", "tune.c"]
PLUGIN_VARIANTS = [(64, 4), (128, 4), (64, 8), (128, 8)]


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n  " + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, jobs=None):
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    steps = []
    objs = []
    for f in CU_SOURCES:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OUT, f + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            steps.append([NVCC] + NVFLAGS + ["-c", src, "-o", obj])
    for f in C_SOURCES:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OUT, f + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            steps.append([CC] + CFLAGS + ["-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        for out in ex.map(_run, steps):
            if verbose and out.strip():
                print(out)
    lib = os.path.join(OUT, "libsgmgb.so")
    if _stale(lib, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", lib] + objs + ["-Xcompiler", "-fPIC", "-lpthread", "-lm"])
    for D, P in PLUGIN_VARIANTS:
        so = os.path.join(OUT, "libsgm_gb300_d%d_p%d.so" % (D, P))
        src = os.path.join(CSRC, "sgm_gb300.c")
        if _stale(so, [src, lib] + headers):
            _run([CC] + CFLAGS + ["-shared", "-DSGM_D=%d" % D, "-DSGM_PATHS=%d" % P, src, "-o", so,
                                  "-L" + OUT, "-lsgmgb", "-Wl,-rpath,$ORIGIN"])
    cli = os.path.join(OUT, "sgmgb_cli")
    src = os.path.join(CSRC, "sgmgb_cli.c")
    if os.path.exists(src) and _stale(cli, [src, lib] + headers):
        _run([CC] + CFLAGS + [src, "-o", cli, "-L" + OUT, "-lsgmgb", "-Wl,-rpath,$ORIGIN", "-lm"])
    return lib


def clean():
    shutil.rmtree(OUT, ignore_errors=True)


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
