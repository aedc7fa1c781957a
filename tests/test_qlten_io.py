"""The .qlten stream format against files written by the reference's own QLTensor stream
operator (tests/golden/qlten/*.qlten; the tensors themselves are in qlten_io.npz).

CPU: parse (every hash checked) and read into host memory; write back byte-identical.
GPU: the device-direct read and write round trip."""
import os

import numpy as np
import pytest

from tensortoolkit_gb300 import capi
from tensortoolkit_gb300.qlten_io import read_qlten_host, write_qlten_host
from tensortoolkit_gb300.tensor import BSTensor, same_topology

HERE = os.path.dirname(os.path.abspath(__file__))
QDIR = os.path.join(HERE, "golden", "qlten")
FILES = [("u_psi", "U1QN", "f64"), ("u_lenv", "U1QN", "f64"), ("f_psi", "fU1U1QN", "c128"),
         ("u_scalar", "U1QN", "f64")]


def _ref(golden, tag):
    rec = golden("qlten_io")
    return BSTensor.from_record(rec, tag)


@pytest.mark.parametrize("tag,qn,dtype", FILES)
def test_read_matches_reference(golden, tag, qn, dtype):
    t = read_qlten_host(os.path.join(QDIR, tag + ".qlten"), qn, dtype)
    ref = _ref(golden, tag)
    if ref.rank:
        assert same_topology(t, ref)
        assert all(a.same_space(b) for a, b in zip(t.legs, ref.legs))
    assert np.array_equal(t.data, ref.data)


@pytest.mark.parametrize("tag,qn,dtype", FILES)
def test_write_is_byte_identical(tmp_path, tag, qn, dtype):
    src = os.path.join(QDIR, tag + ".qlten")
    t = read_qlten_host(src, qn, dtype)
    out = str(tmp_path / (tag + ".qlten"))
    write_qlten_host(out, t)
    with open(src, "rb") as a, open(out, "rb") as b:
        assert a.read() == b.read()


def test_wrong_quantum_number_type_is_rejected():
    with pytest.raises(capi.QltgError):
        read_qlten_host(os.path.join(QDIR, "u_psi.qlten"), "U1U1QN", "f64")
    with pytest.raises(capi.QltgError):
        read_qlten_host(os.path.join(QDIR, "f_psi.qlten"), "U1QN", "c128")


def test_truncated_file_is_rejected(tmp_path):
    src = open(os.path.join(QDIR, "u_psi.qlten"), "rb").read()
    p = tmp_path / "cut.qlten"
    p.write_bytes(src[: len(src) - 64])
    with pytest.raises(capi.QltgError):
        read_qlten_host(str(p), "U1QN", "f64")


@pytest.mark.gpu
@pytest.mark.parametrize("tag,qn,dtype", FILES)
def test_device_round_trip(gpu, golden, tmp_path, tag, qn, dtype):
    from tensortoolkit_gb300.api import read_qlten, write_qlten
    src = os.path.join(QDIR, tag + ".qlten")
    d = read_qlten(src, qn, dtype)
    ref = _ref(golden, tag)
    assert np.array_equal(d.to_host().data, ref.data)
    out = str(tmp_path / (tag + ".qlten"))
    write_qlten(out, d)
    with open(src, "rb") as a, open(out, "rb") as b:
        assert a.read() == b.read()
