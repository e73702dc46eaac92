"""Build the native library libgiwaxs_gb300.so in-tree with nvcc.

Every CUDA translation unit under csrc/ is compiled for sm_103a only
(-gencode arch=compute_103a,code=sm_103a), in parallel, then linked into
giwaxsim_gb300/_lib/libgiwaxs_gb300.so.  Host code is compiled with
-ffp-contract=off so that no compiler-introduced fused multiply-add changes
the float64 arithmetic that index computations replay.

    python -m giwaxsim_gb300.build [--force] [--verbose-ptxas]
"""
import argparse
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libgiwaxs_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found; the GB300 library needs the CUDA "
                           "13 toolkit")
    return path


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                  if f.endswith(".cu"))


def _stale(srcs):
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = srcs + [os.path.join(CSRC, f) for f in os.listdir(CSRC)
                   if f.endswith((".cuh", ".h"))]
    deps.append(os.path.join(ROOT, "include", "giwaxs_gb300.h"))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose_ptxas=False, quiet=True):
    srcs = sources()
    if not force and not _stale(srcs):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    obj_dir = os.path.join(OUT_DIR, "obj")
    os.makedirs(obj_dir, exist_ok=True)
    common = [nvcc(), "-O3", "-std=c++17", "-lineinfo", *ARCH,
              "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-I", os.path.join(ROOT, "include"), "-I", CSRC]
    if verbose_ptxas:
        common += ["-Xptxas", "-v"]
    procs, objs = [], []
    for s in srcs:
        o = os.path.join(obj_dir, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        procs.append((s, subprocess.Popen(
            common + ["-c", s, "-o", o], stdout=subprocess.PIPE,
            stderr=subprocess.STDOUT, text=True)))
    failed = []
    for s, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((s, out))
        elif out and (verbose_ptxas or not quiet):
            sys.stdout.write(out)
    if failed:
        msg = "\n".join("%s:\n%s" % (s, o) for s, o in failed)
        raise RuntimeError("nvcc failed:\n" + msg)
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.check_call([nvcc(), "-shared", *ARCH, "-o", tmp, *objs])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose-ptxas", action="store_true")
    a = ap.parse_args()
    print(build(force=a.force, verbose_ptxas=a.verbose_ptxas, quiet=False))
