"""Loader of the golden fixtures made by tests/golden/make_golden.py."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def index():
    with open(os.path.join(GOLDEN, "index.json")) as f:
        return json.load(f)


def load(name):
    meta = index()[name]
    data = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    return meta, data


def names():
    return sorted(index().keys())
