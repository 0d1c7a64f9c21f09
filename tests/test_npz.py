"""The library's npz reader and writer on the host (no GPU): archives written
by the library load in numpy bit for bit, archives numpy writes (stored and
deflate-compressed) load through the library, and bad calls return status
codes.  The training checkpoint (cnncrf_train_save / _load) is this writer
and reader; its resume test is tests/test_gpu_train.py."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def L():
    from cnncrf import _lib
    _lib.lib()
    return _lib


def arrays(seed=0):
    rng = np.random.default_rng(seed)
    return {
        "arr_0": rng.standard_normal((100, 3, 3, 3)).astype(np.float32),
        "arr_1": rng.standard_normal(100).astype(np.float32),
        "mom_0": rng.standard_normal((7, 5)).astype(np.float32),
        "scalar": np.array(2.5, np.float32),
        "empty": np.zeros((0, 4), np.float32),
    }


def test_library_archive_loads_in_numpy(L, tmp_path):
    a = arrays()
    path = tmp_path / "w.npz"
    L.npz_write(str(path), a)
    with np.load(path) as z:
        assert sorted(z.files) == sorted(a)
        for k, v in a.items():
            assert z[k].dtype == np.float32 and z[k].shape == v.shape
            assert np.array_equal(z[k], v), k
    for k, v in a.items():  # and through the library's own reader
        got = L.npz_read(str(path), k)
        assert got.shape == v.shape and np.array_equal(got, v), k


@pytest.mark.parametrize("compressed", [False, True])
def test_numpy_archive_loads_in_library(L, tmp_path, compressed):
    a = arrays(1)
    path = tmp_path / "n.npz"
    (np.savez_compressed if compressed else np.savez)(path, **a)
    for k, v in a.items():
        got = L.npz_read(str(path), k)
        assert got.shape == v.shape and np.array_equal(got, v), k


def test_rewrite_replaces_the_file(L, tmp_path):
    path = tmp_path / "r.npz"
    L.npz_write(str(path), {"arr_0": np.ones(3, np.float32)})
    L.npz_write(str(path), {"arr_0": np.full(4, 7.0, np.float32)})
    assert np.array_equal(L.npz_read(str(path), "arr_0"), np.full(4, 7.0, np.float32))
    assert not (tmp_path / "r.npz.tmp").exists()


def test_errors(L, tmp_path):
    import ctypes as C
    path = tmp_path / "e.npz"
    L.npz_write(str(path), {"arr_0": np.ones((2, 3), np.float32)})
    with pytest.raises(L.CnnCrfError) as e:
        L.npz_read(str(path), "arr_9")
    assert e.value.status == L.EIO
    with pytest.raises(L.CnnCrfError) as e:
        L.npz_read(str(tmp_path / "missing.npz"), "arr_0")
    assert e.value.status == L.EIO
    s = (C.c_int64 * 4)()
    nd = C.c_int()
    small = np.empty(5, np.float32)
    st = L.lib().cnncrf_npz_read(str(path).encode(), b"arr_0", s, C.byref(nd), small.ctypes.data_as(C.c_void_p), 5)
    assert st == L.ESHAPE and nd.value == 2 and (s[0], s[1]) == (2, 3)
    np.savez(tmp_path / "f64.npz", arr_0=np.ones(3))  # float64: not a parameter array
    with pytest.raises(L.CnnCrfError) as e:
        L.npz_read(str(tmp_path / "f64.npz"), "arr_0")
    assert e.value.status == L.ESHAPE
    with pytest.raises(L.CnnCrfError) as e:  # a directory that does not exist
        L.npz_write(str(tmp_path / "no" / "x.npz"), {"arr_0": np.ones(1, np.float32)})
    assert e.value.status == L.EIO
