"""Build recipe for libturbotrace.so (sm_103a).

Compiles every ``csrc/*.cu`` with nvcc in parallel and links them into
``turbulence_tracing_gb300/_build/libturbotrace.so``.  Translation units whose
FP64 results must round exactly like numpy are compiled with -fmad=false.
"""
import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libturbotrace.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fno-strict-aliasing",
          "--expt-relaxed-constexpr", "-I", INCLUDE]
NO_FMAD = {"tt_grad.cu", "tt_trace64.cu", "tt_detect.cu"}


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stamp():
    h = hashlib.sha256()
    for f in sorted(os.listdir(CSRC)) + ["../../include/turbotrace.h"]:
        p = os.path.normpath(os.path.join(CSRC, f))
        if os.path.isfile(p):
            h.update(f.encode())
            with open(p, "rb") as fh:
                h.update(fh.read())
    h.update(" ".join(ARCH + COMMON).encode())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def build(force=False, verbose=False, ptxas_info=False):
    os.makedirs(OUT, exist_ok=True)
    stamp_file = os.path.join(OUT, "stamp")
    stamp = _stamp()
    if (not force and os.path.exists(LIB) and os.path.exists(stamp_file)
            and open(stamp_file).read() == stamp):
        return LIB
    cc = nvcc()

    def compile_one(src):
        obj = os.path.join(OUT, src[:-3] + ".o")
        cmd = [cc] + ARCH + COMMON + (["-fmad=false"] if src in NO_FMAD else [])
        if ptxas_info:
            cmd += ["-Xptxas", "-v"]
        cmd += ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
        return obj, r.stderr

    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        results = list(ex.map(compile_one, srcs))
    if verbose or ptxas_info:
        for _, err in results:
            if err:
                sys.stderr.write(err)
    tmp = LIB + ".tmp%d" % os.getpid()
    cuda_lib = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(cc))), "lib64")
    cmd = [cc] + ARCH + ["-shared", "-o", tmp] + [o for o, _ in results] + [
        "-L" + cuda_lib, "-lcufft", "-Xlinker", "-rpath=" + cuda_lib]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    with open(stamp_file, "w") as f:
        f.write(stamp)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))
