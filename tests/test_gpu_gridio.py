"""Grid files written from the device (Grid<T>::save, grid.cpp:135-156) read
back by independent readers: Python's gzip module for .uni and .raw (it
checks the stream's CRC-32 and length), numpy for .npz.  The .uni header is
checked field by field against fileio/iogrids.cpp's UniHeader layout
(id "MNT3", dimX/Y/Z, gridType, elementType, bytesPerElement, info[252],
dimT, timestamp)."""
import gzip
import struct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

m = pytest.importorskip("mantaflow_gb300")


def _grids(shape):
    nx, ny, nz = shape
    s = m.Solver(name="io", gridSize=m.vec3(nx, ny, nz), dim=3 if nz > 1 else 2)
    rng = np.random.default_rng(3)
    out = {}
    r = s.create(m.RealGrid)
    a = rng.random((nz, ny, nx), dtype=np.float32)
    m.copyArrayToGridReal(a, r)
    out["real"] = (r, a, 1, 1, 4)
    v = s.create(m.MACGrid)
    b = rng.random((nz, ny, nx, 3), dtype=np.float32)
    m.copyArrayToGridReal(b, v)
    out["mac"] = (v, b, 4 | 8, 2, 12)
    f = s.create(m.FlagGrid)
    f.initDomain(boundaryWidth=0)
    f.fillGrid()
    out["flags"] = (f, f.numpy(), 2 | 32, 0, 4)
    lv = s.create(m.LevelsetGrid)
    m.copyArrayToGridReal(a - 0.5, lv)
    out["levelset"] = (lv, a - 0.5, 1 | 16, 1, 4)
    return s, out


@pytest.mark.parametrize("shape", [(37, 29, 23), (130, 70, 1), (64, 64, 64)])
def test_save_uni_raw_npz(shape, tmp_path):
    nx, ny, nz = shape
    s, grids = _grids(shape)
    for name, (g, want, gtype, etype, bpe) in grids.items():
        p = tmp_path / (name + ".uni")
        g.save(str(p))
        data = gzip.open(p, "rb").read()
        assert data[:4] == b"MNT3"
        dx, dy, dz, gt, et, bp = struct.unpack("<6i", data[4:28])
        assert (dx, dy, dz, gt, et, bp) == (nx, ny, nz, gtype, etype, bpe), name
        dimT, stamp = struct.unpack("<iQ", data[4 + 276:4 + 288])
        assert dimT == 0 and stamp > 0
        body = np.frombuffer(data[4 + 288:], dtype=want.dtype)
        assert np.array_equal(body, want.reshape(-1)), name
        p = tmp_path / (name + ".raw")
        g.save(str(p))
        assert np.array_equal(np.frombuffer(gzip.open(p, "rb").read(), dtype=want.dtype), want.reshape(-1)), name
        p = tmp_path / (name + ".npz")
        g.save(str(p))
        arr = np.load(p)["arr_0"]
        assert arr.shape == (nz, ny, nx, 3 if want.ndim == 4 else 1)
        assert np.array_equal(arr.reshape(want.shape), want), name
    with pytest.raises(m.MantaError) as e:
        grids["real"][0].save(str(tmp_path / "x.vdb2"))
    assert "filetype not supported" in str(e.value)
