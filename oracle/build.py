"""Build recipe for the CPU oracle shared library (test infrastructure only).

Compiles oracle/*.cpp with g++ into oracle/_build/liboracle.so.  The flags keep
IEEE semantics identical on x86_64 and aarch64: no -march=native, no -ffast-math,
and -ffp-contract=off so no multiply-add is fused.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SOURCES = ["cpo.cpp", "cpo_vp.cpp"]
HEADERS = ["cpo.h", "cpo_vp.h", "cpo_pair.h", "cpo_vpcase.inc"]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(HERE, s) for s in SOURCES] + [os.path.join(HERE, h) for h in HEADERS]
    return any(os.path.exists(d) and os.path.getmtime(d) > t for d in deps)


def build(force=False):
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = [os.path.join(HERE, s) for s in SOURCES if os.path.exists(os.path.join(HERE, s))]
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
           "-pthread", "-o", LIB + ".tmp"] + srcs
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
