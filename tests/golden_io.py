"""Loading helpers for the golden fixtures in tests/golden."""
import ast
import hashlib
import os

import numpy as np

import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


def config(d):
    return {k: ast.literal_eval(v) for k, v in d["cfg"]}


class _Cam:
    def __init__(self, k, p):
        self._k, self._p = k, p

    def intrinsics_array(self):
        return self._k

    def pose_array(self):
        return self._p


def viewset(d, prefix=""):
    ref_cam = _Cam(d[prefix + "ref_intr"], d[prefix + "ref_pose"])
    srcs = list(d[prefix + "srcs"])
    return O.ViewSet(d[prefix + "ref"], srcs, ref_cam, None, source_indices=list(d[prefix + "source_indices"]),
                     all_poses=list(d[prefix + "poses"]), intrinsics=list(d[prefix + "intr"]))


def digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()
