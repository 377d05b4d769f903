"""Build libhdc_gb300.so for sm_103a (GB300) with nvcc, in-tree.

Each .cu / .cpp translation unit under csrc/ is compiled in parallel with
    nvcc -gencode arch=compute_103a,code=sm_103a -lineinfo -O3 -Xcompiler -fPIC
and linked into _build/libhdc_gb300.so.  Object files are rebuilt only when a
source or header is newer.  Usage:  python build.py [--force] [-v]
"""
import concurrent.futures
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libhdc_gb300.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O3,-pthread", "-I" + os.path.join(ROOT, "include"),
          "-I" + CSRC]


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h"))


def _compile(src, force, verbose):
    obj = os.path.join(OUT, os.path.basename(src) + ".o")
    newest = max([os.path.getmtime(src)] + [os.path.getmtime(h) for h in _headers()])
    if not force and os.path.exists(obj) and os.path.getmtime(obj) >= newest:
        return obj
    cmd = [NVCC] + ARCH + COMMON + ["-c", src, "-o", obj + ".tmp"]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    os.replace(obj + ".tmp", obj)
    return obj


def build(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 1))) as ex:
        objs = list(ex.map(lambda s: _compile(s, force, verbose), srcs))
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(o) for o in objs):
        return LIB
    cmd = [NVCC] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + ["-cudart", "static", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(LIB + ".tmp", LIB)
    return LIB


SYNTH_SRC = os.path.join(HERE, "synth", "synth.cpp")
SYNTH_LIB = os.path.join(OUT, "libhdc_synth.so")


def build_synth(force=False):
    """libhdc_synth.so: the seeded synthetic-workload generator (include/hdc_synth.h),
    host C++ only and kept out of libhdc_gb300.so, so that a CPU-only user of the
    workloads (the benchmark's reference arm) maps no GPU library."""
    os.makedirs(OUT, exist_ok=True)
    hdr = os.path.join(ROOT, "include", "hdc_synth.h")
    newest = max(os.path.getmtime(SYNTH_SRC), os.path.getmtime(hdr))
    if not force and os.path.exists(SYNTH_LIB) and os.path.getmtime(SYNTH_LIB) >= newest:
        return SYNTH_LIB
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", "-I" + os.path.join(ROOT, "include"),
                           SYNTH_SRC, "-o", SYNTH_LIB + ".tmp"])
    os.replace(SYNTH_LIB + ".tmp", SYNTH_LIB)
    return SYNTH_LIB


DROPIN = os.path.join(HERE, "dropin")


def build_dropin(dim=1024, kmer=8, window=150, step=10, force=False):
    """The GPU.cuh drop-in (dropin/gpu_dropin.cpp, libhdc_dropin.so), the
    self-check drivers of it and of the encoder.h drop-in (dropin/hvcache/),
    and the GPU propagate-children and identify applications for one
    compile-time configuration, linked against libhdc_gb300.so."""
    lib = build(force=force)
    out = os.path.join(OUT, "dropin_D%d_k%d_L%d_s%d" % (dim, kmer, window, step))
    os.makedirs(out, exist_ok=True)
    so = os.path.join(out, "libhdc_dropin.so")
    exe = os.path.join(out, "selftest")
    srcs = [os.path.join(DROPIN, f) for f in ("gpu_dropin.cpp", "selftest.cpp", "GPU.cuh", "config.h",
                                             "hierarchy.cpp", "hierarchy.h", "propagate_gpu.cpp", "identify_gpu.cpp",
                                             "hvcache/encoder.h", "hvcache/encoder_gpu.cpp",
                                             "hvcache/hvcache_selftest.cpp")]
    newest = max([os.path.getmtime(x) for x in srcs] + [os.path.getmtime(lib)])
    last = os.path.join(out, "identify")  # built last
    if not force and os.path.exists(last) and os.path.getmtime(last) >= newest:
        return out
    defs = ["-DHV_DIM=%d" % dim, "-DKMER_SIZE=%d" % kmer, "-DSEQUENCE_LENGTH=%d" % window, "-DSIM_STEP=%d" % step]
    inc = ["-I" + DROPIN, "-I" + os.path.join(ROOT, "include")]
    rpath = "-Wl,-rpath," + OUT + ":" + out
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared"] + defs + inc +
                          [os.path.join(DROPIN, "gpu_dropin.cpp"), "-L" + OUT, "-lhdc_gb300", rpath, "-o", so])
    # the encoder.h drop-in (its own directory: a build opts in by putting it on the include path)
    hv = os.path.join(DROPIN, "hvcache")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-DNORM_COSINE", "-I" + hv] + defs + inc +
                          [os.path.join(hv, "hvcache_selftest.cpp"), os.path.join(hv, "encoder_gpu.cpp"),
                           "-L" + OUT, "-lhdc_gb300", rpath, "-o", os.path.join(out, "hvcache_selftest")])
    subprocess.check_call(["g++", "-O2", "-std=c++17"] + defs + inc +
                          [os.path.join(DROPIN, "selftest.cpp"), "-L" + out, "-lhdc_dropin", "-L" + OUT,
                           "-lhdc_gb300", rpath, "-o", exe])
    subprocess.check_call(["g++", "-O2", "-std=c++20"] + defs + inc +
                          [os.path.join(DROPIN, "propagate_gpu.cpp"), os.path.join(DROPIN, "hierarchy.cpp"),
                           "-L" + OUT, "-lhdc_gb300", rpath, "-o", os.path.join(out, "propagate-children")])
    subprocess.check_call(["g++", "-O2", "-std=c++20"] + defs + inc +
                          [os.path.join(DROPIN, "identify_gpu.cpp"), os.path.join(DROPIN, "hierarchy.cpp"),
                           "-L" + OUT, "-lhdc_gb300", rpath, "-o", os.path.join(out, "identify")])
    return out


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
    print(build_synth(force="--force" in sys.argv))
