"""Build recipe for the CPU oracle (test infrastructure).

Compiles ``oracle/rf_oracle.c`` twice with gcc/OpenMP into ``oracle/_build/``:
``librf_oracle_f32.so`` (RFO_REAL=float, the FP32 parity target) and
``librf_oracle_f64.so`` (RFO_REAL=double, the FP64 oracle). ``-ffp-contract=off`` keeps
the arithmetic free of fused multiply-adds on every host, so x86 and Arm builds agree.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, '_build')
SRC = os.path.join(HERE, 'rf_oracle.c')

VARIANTS = {'f32': 'float', 'f64': 'double'}


def lib_path(variant: str) -> str:
    return os.path.join(OUT, f'librf_oracle_{variant}.so')


def build(force: bool = False) -> None:
    os.makedirs(OUT, exist_ok=True)
    procs = []
    for variant, real in VARIANTS.items():
        out = lib_path(variant)
        if not force and os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(SRC):
            continue
        cmd = [
            'gcc', '-O3', '-std=gnu11', '-fopenmp', '-fPIC', '-shared', '-ffp-contract=off',
            f'-DRFO_REAL={real}', SRC, '-o', out + '.tmp', '-lm',
        ]
        procs.append((subprocess.Popen(cmd), out))
    for proc, out in procs:
        if proc.wait() != 0:
            raise RuntimeError(f'oracle build failed: {out}')
        os.replace(out + '.tmp', out)


if __name__ == '__main__':
    build(force='--force' in sys.argv)
    print('ok')
