"""CI vector files and the reference's PsociVector layout (host code, no GPU).

Where the reference tree is present, files written by this library are read back by the
reference's own PsociVector (compiled unchanged into oracle/_ref) and vice versa, and the
ASCII files of both writers are compared byte for byte.
"""
import ctypes
import os

import numpy as np
import pytest

from psoci_gb300 import api

from oracle import REFERENCE_TREE as REF_TREE  # noqa: E402


def vecs(nroots=3, n=257, seed=0):
    v = np.random.default_rng(seed).standard_normal((nroots, n))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


@pytest.mark.parametrize("binary", [False, True])
def test_round_trip(tmp_path, gpu_lib, binary):
    v = vecs()
    f = str(tmp_path / "civec")
    api.write_vectors(f, v, binary=binary, title="t")
    r = api.read_vectors(f, v.shape[1], 8, binary=binary)
    assert r.shape == v.shape
    if binary:
        assert np.array_equal(r, v)
    else:
        assert np.abs(r - v).max() <= 5e-15  # 14 decimals


def test_ascii_layout(tmp_path, gpu_lib):
    v = vecs(2, 5)
    f = tmp_path / "civec"
    api.write_vectors(str(f), v, title="title line")
    lines = f.read_text().split("\n")
    assert lines[0] == "5 2" and lines[1] == "18 14"
    assert lines[2] == "1" and len(lines[3]) == 5 * 18
    assert float(lines[3][:18]) == pytest.approx(v[0, 0], abs=1e-14)
    assert lines[4] == "2" and lines[6] == "title line"


@pytest.mark.parametrize("binary", [False, True])
def test_rejects_bad_files(tmp_path, gpu_lib, binary):
    v = vecs()
    f = str(tmp_path / "civec")
    api.write_vectors(f, v, binary=binary)
    with pytest.raises(api.PsociError):  # wrong basis size
        api.read_vectors(f, v.shape[1] + 1, 8, binary=binary)
    data = open(f, "rb").read()
    open(f, "wb").write(data[: len(data) // 2])  # truncated
    with pytest.raises(api.PsociError):
        api.read_vectors(f, v.shape[1], 8, binary=binary)
    with pytest.raises(api.PsociError):
        api.read_vectors(str(tmp_path / "missing"), v.shape[1], 8, binary=binary)


@pytest.mark.skipif(not os.path.isdir(REF_TREE), reason="reference tree not present")
@pytest.mark.parametrize("binary", [False, True])
def test_interoperates_with_reference(tmp_path, gpu_lib, binary):
    import oracle

    oracle.build(ref=True)
    lib = ctypes.CDLL(oracle.REF_SO)
    lib.ref_vec_write.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_long, ctypes.c_int,
                                  ctypes.POINTER(ctypes.c_double), ctypes.c_char_p]
    lib.ref_vec_read.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_long, ctypes.c_int,
                                 ctypes.POINTER(ctypes.c_double)]
    lib.ref_vec_read.restype = ctypes.c_int
    v = vecs(3, 300, seed=4)
    dp = ctypes.POINTER(ctypes.c_double)
    ours, theirs = str(tmp_path / "ours"), str(tmp_path / "theirs")
    # the reference's default title for PsociVector(filename)
    title = "default vector test format "
    api.write_vectors(ours, v, binary=binary, title=title)
    saved = os.dup(1)
    devnull = os.open(os.devnull, os.O_WRONLY)
    os.dup2(devnull, 1)
    try:
        lib.ref_vec_write(theirs.encode(), int(binary), v.shape[1], v.shape[0], v.ctypes.data_as(dp), b"")
        out = np.zeros_like(v)
        n = lib.ref_vec_read(ours.encode(), int(binary), v.shape[1], 8, out.ctypes.data_as(dp))
    finally:
        os.dup2(saved, 1)
        os.close(devnull)
        os.close(saved)
    assert n == 3
    mine = api.read_vectors(theirs, v.shape[1], 8, binary=binary)
    if binary:
        assert np.array_equal(out, v) and np.array_equal(mine, v)
        a, b = open(ours, "rb").read(), open(theirs, "rb").read()
        assert len(a) == len(b)
        # identical except the high half of each root tag, which the reference writes from an int
        hdr = 24
        rec = 8 + 8 * v.shape[1]
        mask = np.ones(len(a), bool)
        for r in range(3):
            mask[hdr + r * rec + 4: hdr + r * rec + 8] = False
        assert (np.frombuffer(a, np.uint8)[mask] == np.frombuffer(b, np.uint8)[mask]).all()
    else:
        assert np.abs(out - v).max() <= 5e-15 and np.abs(mine - v).max() <= 5e-15
        assert open(ours, "rb").read() == open(theirs, "rb").read()
