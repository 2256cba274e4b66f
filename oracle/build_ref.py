"""Build recipe for ``oracle/_ref``: the reference's own OpenCL kernels compiled for the host.

Test infrastructure. The reference (realflare v0.6.4) is Python + OpenCL C; its kernels
cannot run here through OpenCL (no platform). This recipe compiles the kernel sources
**where they lie** in the reference checkout into ``oracle/_ref/librf_ref.so``:

1. each OpenCL program is assembled the way the reference's Python tasks assemble it
   (``raytracing.py:43-52,255-265``, ``rasterizing.py:69-101``, ``starburst.py:22-31``,
   ``aperture.py:27-36``, ``diagram.py:32-43``): host-injected constants and struct
   declarations, then the ``.cl`` files;
2. one mechanical rewrite makes OpenCL C parse as C++: vector literals
   ``(floatN)(a, b, ...)`` become ``make_floatN(a, b, ...)``; nothing else is changed;
3. the result is wrapped in a namespace, followed by ``oracle/ref_harness.inc`` (the
   NDRange driver: one OpenMP loop over work-items per launch), and compiled with
   ``oracle/cl_shim.hpp`` (the OpenCL C built-ins in C++).

The generated ``.cpp`` files and the library go to ``oracle/_ref/`` only (kept out of version
control, but copied with the working tree), so a machine without the reference checkout can
rebuild the library from the generated sources (``build(reference=None)``).

The checkout is the ``reference`` argument, else the ``REALFLARE_REFERENCE`` environment
variable; without either, previously generated sources are compiled.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, '_ref')
LIB = os.path.join(OUT, 'librf_ref.so')

_VEC_LITERAL = re.compile(r'\(\s*(u?(?:char|short|int|long|float|double)(?:2|3|4|8|16))\s*\)\s*\(')

_RAY = """typedef struct { float3 pos; float3 dir; float2 pos_apt; float rrel = 0; float reflectance = 0; } Ray;
"""
_LENS = """typedef struct { float radius = 0; float ior = 0; float height = 0; float center = 0; int coating = 0; float8 coefficients; } LensElement;
"""
_INTERSECTION = """typedef struct { float3 pos; float3 normal; float incident = 0; int hit = 0; } Intersection;
"""
_VERTEX = """typedef struct { float2 pos; float2 uv; float rrel = 0; float reflectance = 0; float intensity = 0; } Vertex;
"""

# (program, prefix emulating the host build, .cl files)
PROGRAMS = {
    'raytracing': (
        _RAY + _LENS + _INTERSECTION + 'const int LAMBDA_MIN = 390;\nconst int LAMBDA_MAX = 730;\n',
        ['raytracing.cl'],
    ),
    'rasterizing': (
        '#define BATCH_PRIMITIVE_COUNT 255\n' + _RAY + _VERTEX
        + '__constant uchar sub_offsets[15] = {0, 1, 0, 1, 2, 0, 3, 4, 1, 6, 2, 5, 0, 3, 7};\n'
        + 'static int BIN_SIZE = 64;\n__constant int LAMBDA_MIN = 390;\n__constant int LAMBDA_MAX = 730;\n',
        ['color.cl', 'rasterizing.cl'],
    ),
    'starburst': (
        '__constant int LAMBDA_MIN = 390;\n__constant int LAMBDA_MAX = 730;\n__constant int LAMBDA_MID = 560.0;\n',
        ['noise.cl', 'geometry.cl', 'color.cl', 'starburst.cl'],
    ),
    'aperture': ('', ['noise.cl', 'geometry.cl', 'aperture.cl']),
    # IntersectionsTask.build (raytracing.py:255-265) and DiagramTask.build (diagram.py:32-43)
    'raytracing_inter': (
        _RAY + _LENS + _INTERSECTION + '#define STORE_INTERSECTIONS\n'
        + 'const int LAMBDA_MIN = 390;\nconst int LAMBDA_MAX = 730;\n',
        ['raytracing.cl'],
    ),
    'diagram': (_RAY + _LENS + _INTERSECTION, ['geometry.cl', 'diagram.cl']),
}


def rewrite(source: str) -> str:
    return _VEC_LITERAL.sub(lambda m: f'make_{m.group(1)}(', source)


def generate(reference: str) -> list:
    cl_dir = os.path.join(reference, 'realflare', 'api', 'tasks', 'cl')
    os.makedirs(OUT, exist_ok=True)
    files = []
    for name, (prefix, sources) in PROGRAMS.items():
        body = prefix
        for src in sources:
            with open(os.path.join(cl_dir, src), encoding='utf-8') as f:
                body += f'#line 1 "{src}"\n' + rewrite(f.read()) + '\n'
        text = (
            '// generated by oracle/build_ref.py from the reference checkout; do not edit\n'
            '#include "../cl_shim.hpp"\n'
            f'namespace rf_ref_{name} {{\n{body}\n}}  // namespace\n'
            f'#define RF_REF_PROGRAM_{name.upper()} 1\n'
            f'namespace rf_ref = rf_ref_{name};\n'
            '#include "../ref_harness.inc"\n'
        )
        path = os.path.join(OUT, f'ref_{name}.cpp')
        old = None
        if os.path.exists(path):
            with open(path, encoding='utf-8') as f:
                old = f.read()
        if old != text:
            with open(path, 'w', encoding='utf-8') as f:
                f.write(text)
        files.append(path)
    return files


def build(reference: str | None = None, force: bool = False) -> str | None:
    """Generate (when the reference checkout exists) and compile. Returns the library path,
    or None when neither the reference nor previously generated sources are available."""
    sources = [os.path.join(OUT, f'ref_{n}.cpp') for n in PROGRAMS]
    reference = reference or os.environ.get('REALFLARE_REFERENCE')
    if reference and os.path.isdir(reference):
        sources = generate(reference)
    elif not all(os.path.exists(s) for s in sources):
        return None
    deps = sources + [os.path.join(HERE, 'cl_shim.hpp'), os.path.join(HERE, 'ref_harness.inc')]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in deps):
        return LIB
    objs, procs = [], []
    for src in sources:
        obj = src[:-4] + '.o'
        cmd = ['g++', '-O3', '-std=gnu++17', '-fopenmp', '-fPIC', '-ffp-contract=off', '-w',
               '-c', src, '-o', obj]
        procs.append(subprocess.Popen(cmd))
        objs.append(obj)
    for p in procs:
        if p.wait() != 0:
            raise RuntimeError('reference oracle build failed')
    subprocess.check_call(['g++', '-shared', '-fopenmp', '-o', LIB + '.tmp'] + objs + ['-lm'])
    os.replace(LIB + '.tmp', LIB)
    return LIB


if __name__ == '__main__':
    print(build(sys.argv[1] if len(sys.argv) > 1 and sys.argv[1] != '--force' else None, force='--force' in sys.argv))
