"""Loading helpers for the committed golden fixtures (tests/golden/*.npz)."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False)


def encoder_cases():
    g = load("encoders")
    for key in g["cases"]:
        key = str(key)
        dt, kind, n, B = key.split("_")
        yield key, np.dtype(dt), kind, int(n[1:]), int(B[1:]), g


def split_streams(blob, sizes):
    offs = np.concatenate([[0], np.cumsum(np.asarray(sizes, np.int64))])
    return offs
