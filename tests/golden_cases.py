"""Loads the reference's golden vectors (tests/golden/reference_vectors.json)
as numpy arrays for the oracle and CUDA parity tests."""
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
NP = {"char": np.int8, "uchar": np.uint8, "short": np.int16, "ushort": np.uint16, "int": np.int32,
      "uint": np.uint32, "long": np.int64, "ulong": np.uint64, "float": np.float32,
      "double": np.float64, "int2": np.int32}


def load():
    with open(os.path.join(HERE, "golden", "reference_vectors.json")) as f:
        return json.load(f)["cases"]


def cases(*kinds):
    return [c for c in load() if c["kind"] in kinds]


def arr(values, dtype):
    a = np.array(values, dtype=NP[dtype])
    return a


def scalar(v, dtype):
    if v == "FLT_MAX":
        return float(np.finfo(np.float32).max)
    if v == "FLT_MIN":
        return float(np.finfo(np.float32).tiny)
    return v


def ids(cs):
    return [c["id"] for c in cs]
