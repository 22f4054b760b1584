"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/rt_oracle.c twice with gcc:
  librt_oracle.so      serial, -O2 -ffp-contract=off (the parity checker)
  librt_oracle_omp.so  same source with -fopenmp (timed CPU baseline)
Both keep the reference's operation order: no fused multiply-add, no
fast-math.  Outputs stay next to the source and are git-ignored.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "rt_oracle.c")
FLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-std=c11", "-Wall"]


def _up_to_date(out):
    return os.path.exists(out) and os.path.getmtime(out) >= max(
        os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "rt_oracle.h")))


def build(force=False):
    outs = []
    for name, extra in (("librt_oracle.so", []), ("librt_oracle_omp.so", ["-fopenmp"])):
        out = os.path.join(HERE, name)
        if force or not _up_to_date(out):
            cmd = ["gcc"] + FLAGS + extra + [SRC, "-o", out + ".tmp", "-lm"]
            subprocess.run(cmd, check=True)
            os.replace(out + ".tmp", out)
        outs.append(out)
    return outs


if __name__ == "__main__":
    print("\n".join(build(force="--force" in sys.argv)))
