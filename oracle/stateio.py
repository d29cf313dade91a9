"""Flatten GO-MELT state trees (lists/dicts of arrays) to and from .npz files.

TEST INFRASTRUCTURE.  The reference keeps its whole simulation state in a list
of four dicts (``Levels``, built by ``SetupLevels``,
``go_melt/computeFunctions.py:115-264``) whose values are arrays, scalars,
lists of arrays and nested dicts.  Golden fixtures store such trees as flat
``.npz`` archives: dict keys are joined with ``.``, list items with ``#i``,
and every list/tuple records its length (and kind) so the tree can be rebuilt.
"""

from __future__ import annotations

import json

import numpy as np


def flatten(tree, prefix: str, out: dict) -> dict:
    if isinstance(tree, dict):
        out[prefix + "@dict"] = np.asarray(json.dumps(sorted(str(k) for k in tree)))
        for k, v in tree.items():
            flatten(v, f"{prefix}.{k}", out)
    elif isinstance(tree, (list, tuple)):
        out[prefix + "@list"] = np.asarray([len(tree), 1 if isinstance(tree, tuple) else 0])
        for i, v in enumerate(tree):
            flatten(v, f"{prefix}#{i}", out)
    elif tree is None:
        out[prefix + "@none"] = np.asarray(0)
    elif isinstance(tree, str):
        out[prefix + "@str"] = np.asarray(tree)
    else:
        out[prefix] = np.array(tree)
    return out


def _rebuild(prefix: str, data: dict):
    if prefix + "@dict" in data:
        keys = json.loads(str(data[prefix + "@dict"]))
        return {k: _rebuild(f"{prefix}.{k}", data) for k in keys}
    if prefix + "@list" in data:
        n, is_tuple = (int(x) for x in data[prefix + "@list"])
        items = [_rebuild(f"{prefix}#{i}", data) for i in range(n)]
        return tuple(items) if is_tuple else items
    if prefix + "@none" in data:
        return None
    if prefix + "@str" in data:
        return str(data[prefix + "@str"])
    return np.array(data[prefix])


def unflatten(data, prefix: str):
    """Rebuild the tree stored under ``prefix`` from an npz mapping."""
    return _rebuild(prefix, dict(data) if not isinstance(data, dict) else data)


def load(path):
    with np.load(path, allow_pickle=False) as z:
        return {k: z[k] for k in z.files}
