"""Copy the reference's own benchmark project into ``tests/golden/``.

``benchmark/nikon_ai_50_135mm/project.json`` of the reference is the project its published
timings were measured on (``benchmark/nikon_ai_50_135mm/report_v0.5.0.md``): the Nikon AI
50-135 mm prescription (``$RES/model/Nikon/ai_50_135mm.json``, bundled under
``realflare_gb300/resources/model``), 1920 x 1080, anti-aliasing 4, 5 wavelengths with 8
sub-steps, a 129 x 129 grid and 50 % ghost culling. The file is re-serialised unchanged.

Usage: ``python tests/golden/make_benchmark_project.py <reference checkout>`` (or set
``REALFLARE_REFERENCE``).
"""
from __future__ import annotations

import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, 'nikon_ai_50_135mm.project.json')


def main(reference: str) -> None:
    with open(os.path.join(reference, 'benchmark', 'nikon_ai_50_135mm', 'project.json'), encoding='utf-8') as f:
        data = json.load(f)
    with open(OUT, 'w', encoding='utf-8') as f:
        json.dump(data, f, indent=1)
        f.write('\n')
    print(OUT)


if __name__ == '__main__':
    checkout = sys.argv[1] if len(sys.argv) > 1 else os.environ.get('REALFLARE_REFERENCE')
    if not checkout:
        sys.exit('usage: make_benchmark_project.py <reference checkout> (or set REALFLARE_REFERENCE)')
    main(checkout)
