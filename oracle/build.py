"""Build recipe for the oracle (test infrastructure only).

Compiles the C++ restatement of the reference's hot path into
``oracle/_build/liboracle.so`` (loaded by the tests and the CPU baseline
through ctypes) and ``oracle/_build/kat`` (the reference's known-answer tests
restated against it).  Uses ``g++`` directly so that it runs on any host with
a C++17 compiler, x86_64 or aarch64.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
CXXFLAGS = ["-std=c++17", "-O2", "-fPIC", "-pthread", "-Wall", "-Wno-unused-function"]


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    hdrs = [os.path.join(HERE, "oracle.hpp"), os.path.join(HERE, "..", "include", "gprt.h")]
    lib = os.path.join(OUT, "liboracle.so")
    kat = os.path.join(OUT, "kat")
    jobs = []
    src = os.path.join(HERE, "oracle.cpp")
    if _stale(lib, [src] + hdrs):
        jobs.append(["g++", *CXXFLAGS, "-shared", "-o", lib, src])
    ksrc = os.path.join(HERE, "kat.cpp")
    if _stale(kat, [ksrc] + hdrs):
        jobs.append(["g++", *CXXFLAGS, "-o", kat, ksrc])
    procs = [subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT) for j in jobs]
    for j, p in zip(jobs, procs):
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("oracle build failed: %s\n%s" % (" ".join(j), out.decode()))
        if verbose and out:
            print(out.decode())
    return lib, kat


if __name__ == "__main__":
    print(build(verbose=True))
    sys.exit(0)
