"""Regenerate the data tables under ``realflare_gb300/resources`` from the reference checkout.

The render path needs two public data tables at run time:

* ``schott.json``: the Schott glass catalogue (name, n_d, V_d and the six Sellmeier
  coefficients of the ``formula 2`` entry) from the refractiveindex.info YAML files that the
  reference ships in ``realflare/resources/glass/schott`` (public domain, CC0). The parse
  follows ``realflare/api/glass.py:32-70``: the first ``formula 2`` entry, its coefficients
  without the leading 0, and ``nd``/``Nd`` plus ``vd``/``Vd`` from ``SPECS``; files without
  them are skipped. Files are stored in sorted file-name order, the order the reference's
  own test relies on (``tests/glass.py:15-30`` expects BAFN6 first).
* ``ciexyz.csv``: the CIE 2006 10-degree colour matching table of
  ``realflare/utils/ciexyz.py:4-406`` (wavelength nm, X, Y, Z).
* ``model/<maker>/<name>.json``: the seven published lens prescriptions the reference
  ships in ``realflare/resources/model`` (patent data), re-serialised unchanged, so that a
  project's ``$RES/model/...`` lens path resolves here as it does in the reference
  (``realflare/storage.py:80``).

Usage: ``python realflare_gb300/resources/make_resources.py <reference checkout>`` (or the
checkout in the ``REALFLARE_REFERENCE`` environment variable).
PyYAML is not needed: only the two fields above are read, line by line.
"""
from __future__ import annotations

import ast
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def _parse_glass_yaml(text: str):
    coefficients = None
    nd = vd = None
    in_formula2 = False
    for raw in text.splitlines():
        line = raw.strip()
        if line.startswith('- type:'):
            in_formula2 = line.split(':', 1)[1].strip() == 'formula 2' and coefficients is None
            continue
        if in_formula2 and line.startswith('coefficients:'):
            values = line.split(':', 1)[1].split()
            coefficients = [float(v) for v in values[1:]]
            in_formula2 = False
            continue
        key, _, value = line.partition(':')
        if key in ('nd', 'Nd') and nd is None and value.strip():
            nd = float(value)
        elif key in ('vd', 'Vd') and vd is None and value.strip():
            vd = float(value)
    if not coefficients or not nd or not vd:
        return None
    return nd, vd, coefficients


def make_glass_table(reference: str) -> list[dict]:
    directory = os.path.join(reference, 'realflare', 'resources', 'glass', 'schott')
    table = []
    for file_name in sorted(os.listdir(directory)):
        if not file_name.endswith(('.yml', '.yaml')):
            continue
        with open(os.path.join(directory, file_name), encoding='utf-8') as f:
            parsed = _parse_glass_yaml(f.read())
        if parsed is None:
            continue
        nd, vd, coefficients = parsed
        table.append(
            {
                'name': os.path.splitext(file_name)[0],
                'manufacturer': 'schott',
                'n': nd,
                'v': vd,
                'coefficients': coefficients,
            }
        )
    return table


def make_cie_table(reference: str) -> list[list[float]]:
    path = os.path.join(reference, 'realflare', 'utils', 'ciexyz.py')
    with open(path, encoding='utf-8') as f:
        tree = ast.parse(f.read())
    for node in tree.body:
        if isinstance(node, ast.Assign) and node.targets[0].id == 'CIEXYZ':
            return ast.literal_eval(node.value)
    raise ValueError('CIEXYZ table not found')


def copy_lens_models(reference: str) -> list[str]:
    source = os.path.join(reference, 'realflare', 'resources', 'model')
    written = []
    for maker in sorted(os.listdir(source)):
        if not os.path.isdir(os.path.join(source, maker)):
            continue
        for file_name in sorted(os.listdir(os.path.join(source, maker))):
            if not file_name.endswith('.json'):
                continue
            with open(os.path.join(source, maker, file_name), encoding='utf-8') as f:
                data = json.load(f)
            os.makedirs(os.path.join(HERE, 'model', maker), exist_ok=True)
            with open(os.path.join(HERE, 'model', maker, file_name), 'w', encoding='utf-8') as f:
                json.dump(data, f, indent=2)
                f.write('\n')
            written.append(f'{maker}/{file_name}')
    return written


def main(reference: str) -> None:
    glasses = make_glass_table(reference)
    with open(os.path.join(HERE, 'schott.json'), 'w', encoding='utf-8') as f:
        json.dump(glasses, f, indent=0)
    cie = make_cie_table(reference)
    with open(os.path.join(HERE, 'ciexyz.csv'), 'w', encoding='utf-8') as f:
        f.write('# wavelength_nm,X,Y,Z (CIE 2006 10 degree)\n')
        for row in cie:
            f.write(','.join(repr(v) for v in row) + '\n')
    models = copy_lens_models(reference)
    print(f'{len(glasses)} glasses, {len(cie)} CIE rows, {len(models)} lens models')


if __name__ == '__main__':
    checkout = sys.argv[1] if len(sys.argv) > 1 else os.environ.get('REALFLARE_REFERENCE')
    if not checkout:
        sys.exit('usage: make_resources.py <reference checkout> (or set REALFLARE_REFERENCE)')
    main(checkout)
