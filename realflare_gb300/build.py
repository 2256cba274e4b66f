"""In-tree build of the CUDA library ``realflare_gb300/librealflare_gb300.so`` for sm_103a.

Each translation unit under ``csrc/`` is compiled by nvcc in parallel and linked into one
shared library that Python loads with ctypes (no torch extension: the C ABI takes plain
pointers). Object files go to ``realflare_gb300/_build/``.

The quad/vertex setup is compiled without fused multiply-add contraction so that its
outputs equal the oracle's bit for bit; the trace likewise unless RF_TRACE_FMAD=1 (the
trace's positions then differ from the reference's by a few ulps); every other unit uses
nvcc's default contraction. The trace, its adjoint and the rasteriser flush denormals
(-ftz=true): their values are never denormal in practice, and the flag drops the denormal
handling around reciprocals, square roots and divisions (the trace's outputs stay
bit-identical).
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
BUILD = os.path.join(HERE, '_build')
LIB = os.path.join(HERE, 'librealflare_gb300.so')
STATS_LIB = os.path.join(HERE, 'librealflare_gb300_stats.so')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']

UNITS = {
    'rf_api.cu': [],
    'rf_trace.cu': ['-ftz=true'] + ([] if os.environ.get('RF_TRACE_FMAD') == '1' else ['-fmad=false']),
    # the accurate trace's double arithmetic is the oracle's double build operation for operation
    'rf_trace_accurate.cu': ['-ftz=true', '-fmad=false'],
    'rf_quad.cu': ['-fmad=false'],
    'rf_sort.cu': [],
    'rf_bin.cu': [],
    'rf_raster.cu': ['-ftz=true'],
    'rf_fft.cu': [],
    'rf_image.cu': [],
    'rf_batch.cu': [],
    # the adjoint re-traces rays: it must use the trace's arithmetic
    'rf_adjoint.cu': ['-ftz=true'] + ([] if os.environ.get('RF_TRACE_FMAD') == '1' else ['-fmad=false']),
    'rf_diagram.cu': ['-ftz=true'] + ([] if os.environ.get('RF_TRACE_FMAD') == '1' else ['-fmad=false']),
}


def nvcc() -> str:
    for cand in (os.environ.get('NVCC'), '/usr/local/cuda/bin/nvcc', 'nvcc'):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return 'nvcc'


def _stale(target: str, deps: list) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, stats: bool = False) -> str:
    """Build the library; ``stats`` builds ``librealflare_gb300_stats.so`` instead, whose
    k_raster also counts its record iterations and fragments (``rf_raster_stats``)."""
    build_dir = os.path.join(BUILD, 'stats') if stats else BUILD
    lib = STATS_LIB if stats else LIB
    units = dict(UNITS)
    if stats:
        units['rf_raster.cu'] = units['rf_raster.cu'] + ['-DRF_RASTER_STATS=1']
    os.makedirs(build_dir, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith('.cuh')]
    headers.append(os.path.join(HERE, '..', 'include', 'realflare_gb300.h'))
    flags_file = os.path.join(build_dir, 'flags.txt')
    flag_sig = repr(sorted(units.items()))
    if not os.path.exists(flags_file) or open(flags_file).read() != flag_sig:
        force = True
    objs, procs = [], []
    for unit, extra in units.items():
        src = os.path.join(CSRC, unit)
        obj = os.path.join(build_dir, unit.replace('.cu', '.o'))
        objs.append(obj)
        if not force and not _stale(obj, [src] + headers):
            continue
        cmd = [nvcc(), *ARCH, '-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC,-ffp-contract=off',
               '-Xptxas', '-warn-spills', *extra, '-c', src, '-o', obj]
        if verbose:
            cmd.insert(-4, '-Xptxas=-v')
        procs.append((subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT), unit))
    failed = []
    for proc, unit in procs:
        out, _ = proc.communicate()
        if out and (verbose or proc.returncode != 0):
            sys.stderr.write(out.decode(errors='replace'))
        if proc.returncode != 0:
            failed.append(unit)
    if failed:
        raise RuntimeError(f'nvcc failed for {failed}')
    if force or procs or _stale(lib, objs):
        cmd = [nvcc(), *ARCH, '-shared', '-o', lib + '.tmp', *objs, '-lcudart']
        subprocess.check_call(cmd)
        os.replace(lib + '.tmp', lib)
    with open(flags_file, 'w') as f:
        f.write(flag_sig)
    return lib


if __name__ == '__main__':
    print(build(force='--force' in sys.argv, verbose='-v' in sys.argv, stats='--stats' in sys.argv))
