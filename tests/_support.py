"""Test helpers: the oracle (CPU checker) and the CUDA library side by side."""
import ctypes
import os

import numpy as np

import __graft_entry__ as ge
import weldform_gb300 as wf

_ORACLE = None


def oracle_lib():
    """Load (building if needed) the CPU oracle library."""
    global _ORACLE
    if _ORACLE is None:
        path = os.path.join(ge.ORACLE_BUILD, "libwf_oracle.so")
        if not os.path.exists(path):
            ge.build_oracle()
        _ORACLE = wf.bind(ctypes.CDLL(path), "wfo_")
    return _ORACLE


def oracle_domain(**kw):
    return wf.Domain(lib=oracle_lib(), prefix="wfo_", **kw)


def gpu_domain():
    return wf.Domain()


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b)
    if nb == 0.0:
        return float(np.linalg.norm(a - b))
    return float(np.linalg.norm(a - b) / nb)


def rows(off, idx):
    return [list(idx[off[i]:off[i + 1]]) for i in range(len(off) - 1)]
