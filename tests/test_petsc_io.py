"""PETSc binary Vec files: the byte layout VecView writes (big-endian classid
1211214, int32 length, big-endian doubles) and round trips."""
import os
import struct

import numpy as np


def test_layout_matches_petsc_binary_vec(sbp, tmp_path):
    v = np.array([1.5, -2.0, 3.25e-300, np.pi])
    path = os.path.join(tmp_path, "v.bin")
    sbp.write_petsc_vec(path, v)
    raw = open(path, "rb").read()
    assert raw[:8] == struct.pack(">ii", 1211214, 4)
    assert raw[8:] == struct.pack(">4d", *v)


def test_round_trip_and_errors(sbp, tmp_path):
    rng = np.random.default_rng(0)
    v = rng.standard_normal(3 * 37 * 29)
    path = os.path.join(tmp_path, "state")
    sbp.write_petsc_vec(path, v)
    assert np.array_equal(sbp.read_petsc_vec(path), v)
    empty = os.path.join(tmp_path, "empty")
    sbp.write_petsc_vec(empty, np.zeros(0))
    assert sbp.read_petsc_vec(empty).size == 0
    bad = os.path.join(tmp_path, "bad")
    open(bad, "wb").write(b"\x00" * 16)
    try:
        sbp.read_petsc_vec(bad)
        raise AssertionError("a file without the Vec classid was accepted")
    except sbp.SbpError as e:
        assert e.code == sbp.ERR_INVALID
