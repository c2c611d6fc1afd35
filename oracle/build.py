"""Compiles the oracle's C restatement into oracle/_build/libwavey_oracle.so.

Test infrastructure only (see oracle/__init__.py).  -ffp-contract=off keeps
every product and sum separately rounded, as the reference's Rust code and
the FP32 shader order require; GCC would otherwise fuse them on aarch64.
"""
from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build" / "libwavey_oracle.so"


def build(force: bool = False) -> Path:
    srcs = [HERE / "fdtd_oracle.c", HERE / "fp16_oracle.c", HERE / "ir_oracle.c"]
    if not force and OUT.exists() and all(OUT.stat().st_mtime >= s.stat().st_mtime for s in srcs):
        return OUT
    OUT.parent.mkdir(exist_ok=True)
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", *map(str, srcs), "-o", str(OUT),
           "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stderr}")
    return OUT


if __name__ == "__main__":
    print(build(force=True))
