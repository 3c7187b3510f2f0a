"""Loading helpers for the golden fixtures written by tests/golden/gen_golden.py."""
import glob
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    d = {k: z[k] for k in z.files}
    d["config"] = json.loads(bytes(d["config"]).decode())
    d["iters"] = int(d["iters"])
    d["now_t"] = float(d["now_t"])
    return d
