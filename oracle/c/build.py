"""Compile oracle/c/flare_oracle.c into oracle/_ref/libflare_oracle.so
(gcc -O3 -fopenmp; portable flags only, no -march)."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(os.path.dirname(HERE), "_ref", "libflare_oracle.so")


def build(force=False):
    src = os.path.join(HERE, "flare_oracle.c")
    if not force and os.path.exists(OUT) and os.path.getmtime(OUT) >= os.path.getmtime(src):
        return OUT
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    subprocess.run(["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off",
                    src, "-o", OUT + ".tmp", "-lm"], check=True)
    os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build(force=True))
