"""Argument checks the Python mirror makes before it touches a device (no GPU needed)."""
import numpy as np
import pytest

from tensortoolkit_gb300 import workloads
from tensortoolkit_gb300.api import AxisProjectPlan, LinearCombinePlan, _contiguous_axes


@pytest.fixture(scope="module")
def cfg1():
    return workloads.config1(5)


def test_linear_combine_coefficients(cfg1):
    a, _ = cfg1
    with pytest.raises(ValueError):                 # one coefficient per tensor
        LinearCombinePlan([1.0, 2.0], [a])
    with pytest.raises(ValueError):                 # complex coefficient, real tensors
        LinearCombinePlan([1.0 + 2.0j], [a])
    with pytest.raises(ValueError):                 # complex beta, real tensors
        LinearCombinePlan([1.0], [a], beta=0.5j, res=a)


def test_project_kept_lists(cfg1):
    a, _ = cfg1
    with pytest.raises(ValueError):                 # one kept list per sector
        AxisProjectPlan(a, 0, [[0]] * (a.legs[0].nsct + 1))


def test_contiguous_axes_cyclic():
    # ContractContiguousAxes(A rank 4, B rank 3, a_start 3, b_start 2, n 2): A's axes 3, 0 with
    # B's 2, 0; saved legs in cyclic order from the end of each range
    axa, axb, sa, sb = _contiguous_axes(4, 3, 3, 2, 2)
    assert (axa, axb, sa, sb) == ([3, 0], [2, 0], [1, 2], [1])
    assert np.array_equal(sorted(axa + sa), [0, 1, 2, 3]) and sorted(axb + sb) == [0, 1, 2]
