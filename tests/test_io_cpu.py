"""AMReX-format files of the library (CPU only: host writer and reader, no
device work): a two-level plotfile written by mbg_write_plotfile and read back
by an independent parser (tests/plotfile.py) field for field, and VisMF
multifab round trips, with and without ghost cells in the file."""
import os

import numpy as np
import pytest

import plotfile


def _levels():
    lev0 = np.array([[0, 0, 0, 7, 7, 3], [8, 0, 0, 15, 7, 3], [0, 8, 0, 15, 11, 3]], dtype=np.int32)
    lev1 = np.array([[4, 4, 0, 11, 11, 7], [12, 4, 0, 19, 11, 7]], dtype=np.int32)
    return [lev0, lev1]


def _data(boxes, ncomp, seed):
    rng = np.random.default_rng(seed)
    vol = int(np.prod(boxes[:, 3:] - boxes[:, :3] + 1, axis=1).sum())
    return rng.standard_normal(vol * ncomp)


def test_plotfile_round_trip(tmp_path):
    import marbles_gb300 as M
    levels = _levels()
    names = ["rho", "vel_x", "vel_y", "vel_z", "is_fluid"]
    data = [_data(b, len(names), 7 + l) for l, b in enumerate(levels)]
    path = str(tmp_path / "plt00010")
    M.write_plotfile(path, levels, data, names, n_cell=[16, 12, 4], prob_lo=[0.0, 0.0, -1.0],
                     prob_hi=[16.0, 12.0, 3.0], time=10.0, level_steps=[10, 20])
    pf = plotfile.read_plotfile(path)
    assert pf["names"] == names
    assert pf["time"] == 10.0 and pf["finest_level"] == 1 and pf["ref_ratio"] == [2]
    assert pf["domains"] == [[0, 0, 0, 15, 11, 3], [0, 0, 0, 31, 23, 7]]
    assert pf["level_steps"] == [10, 20]
    assert pf["dx"] == [[1.0, 1.0, 1.0], [0.5, 0.5, 0.5]]
    for lev, b in enumerate(levels):
        got = pf["levels"][lev]
        assert (got["boxes"] == b).all()
        off = 0
        for n, box in enumerate(b):
            nx, ny, nz = box[3:] - box[:3] + 1
            vol = nx * ny * nz
            ref = data[lev][off:off + vol * len(names)].reshape(len(names), nz, ny, nx)
            assert np.array_equal(got["data"][n], ref)
            assert np.array_equal(got["mins"][n], ref.reshape(len(names), -1).min(axis=1))
            assert np.array_equal(got["maxs"][n], ref.reshape(len(names), -1).max(axis=1))
            off += vol * len(names)
        # physical extents of each box
        dx = 1.0 / 2 ** lev
        for n, box in enumerate(b):
            for d in range(3):
                lo = [0.0, 0.0, -1.0][d]
                assert got["phys"][3 * n + d] == [lo + box[d] * dx, lo + (box[d + 3] + 1) * dx]


def test_multifab_round_trip(tmp_path):
    import marbles_gb300 as M
    boxes = _levels()[0]
    d = _data(boxes, 27, 3)
    prefix = str(tmp_path / "f_00")
    M.write_multifab(prefix, boxes, 27, d)
    assert os.path.exists(prefix + "_H") and os.path.exists(prefix + "_D_00000")
    back = M.read_multifab(prefix, boxes, 27)
    assert np.array_equal(back, d)
    b, nc, ng, arrs, _, _ = plotfile.read_multifab(prefix)
    assert (b == boxes).all() and nc == 27 and ng == 0


def test_multifab_reader_keeps_valid_region_of_grown_fabs(tmp_path):
    """A VisMF file written with 3 ghost cells (as the reference's
    checkpoints are): the reader returns the valid cells."""
    import marbles_gb300 as M
    boxes = _levels()[0]
    ng, nc = 3, 2
    rng = np.random.default_rng(5)
    prefix = str(tmp_path / "g_00")
    valid = []
    with open(prefix + "_D_00000", "wb") as fd:
        offs = []
        for b in boxes:
            lo, hi = b[:3] - ng, b[3:] + ng
            n = hi - lo + 1
            a = rng.standard_normal((nc, n[2], n[1], n[0]))
            valid.append(a[:, ng:-ng, ng:-ng, ng:-ng].reshape(-1))
            offs.append(fd.tell())
            fd.write(("FAB ((8, (64 11 52 0 1 12 0 1023)),(8, (1 2 3 4 5 6 7 8)))((%d,%d,%d) (%d,%d,%d) (0,0,0)) %d\n"
                      % (lo[0], lo[1], lo[2], hi[0], hi[1], hi[2], nc)).encode())
            fd.write(a.astype("<f8").tobytes())
    with open(prefix + "_H", "w") as h:
        h.write("1\n0\n%d\n%d\n(%d 0\n" % (nc, ng, len(boxes)))
        for b in boxes:
            h.write("((%d,%d,%d) (%d,%d,%d) (0,0,0))\n" % tuple(b))
        h.write(")\n%d\n" % len(boxes))
        for o in offs:
            h.write("FabOnDisk: g_00_D_00000 %d\n" % o)
        h.write("\n%d,%d\n" % (len(boxes), nc) + "0,0,\n" * len(boxes))
        h.write("\n%d,%d\n" % (len(boxes), nc) + "0,0,\n" * len(boxes))
    back = M.read_multifab(prefix, boxes, nc)
    assert np.array_equal(back, np.concatenate(valid))


def test_multifab_reader_rejects_other_grids(tmp_path):
    import marbles_gb300 as M
    boxes = _levels()[0]
    prefix = str(tmp_path / "f_00")
    M.write_multifab(prefix, boxes, 1, _data(boxes, 1, 1))
    other = boxes.copy()
    other[0, 3] -= 1
    with pytest.raises(M.MbgError, match="differs"):
        M.read_multifab(prefix, other, 1)
