"""Build the C restatement (oracle/hdc_oracle.c) into oracle/_build/liboracle.so,
and, when the reference checkout is present, the compiled reference drivers
(oracle/build_ref.sh -> oracle/_ref/).  Test infrastructure only."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
# the reference checkout: $REF_ROOT, else a directory "reference" beside this repository
REF_ROOT = os.environ.get("REF_ROOT", os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))


def build_oracle(force=False):
    src = os.path.join(HERE, "hdc_oracle.c")
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    tmp = LIB + ".tmp"
    subprocess.check_call(["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-pthread", src, "-o", tmp, "-lm"])
    os.replace(tmp, LIB)
    return LIB


def reference_available():
    return os.path.exists(os.path.join(REF_ROOT, "src", "HV.cpp"))


def build_ref(dim, k, window, step):
    """Path of the compiled reference driver for one configuration, or None
    when the reference checkout is absent."""
    out = os.path.join(HERE, "_ref", f"ref_driver_D{dim}_k{k}_L{window}_s{step}")
    if not reference_available():
        return out if os.path.exists(out) else None
    subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh"), str(dim), str(k), str(window), str(step)],
                          stdout=subprocess.DEVNULL)
    return out


if __name__ == "__main__":
    print(build_oracle(force=True))
