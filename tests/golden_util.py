import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name: str):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))
