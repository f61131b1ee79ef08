"""Load the golden fixtures of tests/golden/ (generated from the reference's
own kernels by tests/golden/make_golden.py)."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)
