"""TEST INFRASTRUCTURE ONLY: builds the oracle's small C helper.

Compiles oracle/oracle_fma.c into oracle/_build/liboracle_fma.so with gcc and
-ffp-contract=off (no compiler-introduced fusions).  Called from
__graft_entry__.build() and lazily by the oracle itself; builds for whatever
host it runs on (x86_64 here, aarch64 on the GPU host).
"""
import os
import subprocess
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "oracle_fma.c")
OUT_DIR = os.path.join(HERE, "_build")
OUT = os.path.join(OUT_DIR, "liboracle_fma.so")


_LOCK = threading.Lock()


def build(force: bool = False) -> str:
    with _LOCK:  # threads of one process share the temporary file name
        return _build(force)


def _build(force):
    if (not force and os.path.exists(OUT)
            and os.path.getmtime(OUT) >= os.path.getmtime(SRC)):
        return OUT
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = OUT + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
                           "-o", tmp, SRC, "-lm"])
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force=True))
