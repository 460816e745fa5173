"""Builds the GB300 rendering library libgprt.so in-tree.

Every translation unit under csrc/ is compiled for sm_103a in parallel with
nvcc (one -gencode, -lineinfo) and linked into
``go-progressive-raytracer_gb300/_build/libgprt.so`` with the CUDA runtime
linked statically, so the library carries no runtime dependency beyond the
driver.  Run ``python go-progressive-raytracer_gb300/build.py``.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libgprt.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
           "-Xcompiler", "-pthread"]


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".cu", ".cpp")))


def headers():
    hs = [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(HERE, "..", "include", "gprt.h"))
    return hs


def _newer(a, deps):
    if not os.path.exists(a):
        return True
    t = os.path.getmtime(a)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, extra_flags=()):
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()
    hs = headers()
    objs, jobs = [], []
    for s in sources():
        o = os.path.join(OUT, os.path.basename(s) + ".o")
        objs.append(o)
        if _newer(o, [s] + hs):
            cmd = [cc, *ARCH, *NVFLAGS, *extra_flags, "-c", s, "-o", o]
            if verbose:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    procs = [(j, subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)) for j in jobs]
    logs = []
    for j, p in procs:
        out, _ = p.communicate()
        txt = out.decode(errors="replace")
        if p.returncode != 0:
            raise RuntimeError("nvcc failed: %s\n%s" % (" ".join(j), txt))
        logs.append(txt)
    if jobs or not os.path.exists(LIB):
        link = [cc, *ARCH, "-shared", "-Xcompiler", "-pthread", "-o", LIB, *objs, "-lpthread"]
        p = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if p.returncode != 0:
            raise RuntimeError("link failed: %s\n%s" % (" ".join(link), p.stdout.decode(errors="replace")))
    if verbose:
        print("\n".join(l for l in logs if l))
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
