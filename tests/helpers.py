"""Comparison helpers shared by the GPU tests.

A task's optimum is the record without its ``route`` (which search path
settled it): two runs that settle the same permutation by different paths
must agree on every other field.
"""
import numpy as np

from dual_threshold_optimization_gb300._lib import OPTIMUM_FIELDS


def same_records(a, b):
    """Structured record arrays equal in every optimum field."""
    if a.shape != b.shape:
        return False
    return all(np.array_equal(a[f], b[f]) for f in OPTIMUM_FIELDS)


def optimum(d):
    """The optimum fields of a record dict (a result's ``unpermuted``)."""
    return {k: d[k] for k in OPTIMUM_FIELDS if k in d}
