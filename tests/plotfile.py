"""Minimal reader of AMReX plotfiles and VisMF multifabs (test infrastructure).

Parses the HyperCLaw-V1.1 Header, each level's VisMF header (Cell_H) and
the FAB records of the data files, independently of the library's writer.
"""
import os
import re

import numpy as np

BOX = re.compile(r"\(\((-?\d+),(-?\d+),(-?\d+)\) \((-?\d+),(-?\d+),(-?\d+)\) \((\d+),(\d+),(\d+)\)\)")


def read_multifab(prefix):
    """Returns (boxes (nbox, 6), ncomp, ngrow, [array (ncomp, nz, ny, nx)
    per box over the box grown by ngrow], mins, maxs)."""
    text = open(prefix + "_H").read()
    lines = text.split("\n")
    version, how, ncomp = int(lines[0]), int(lines[1]), int(lines[2])
    assert version == 1 and how == 0
    ngrow = int(lines[3])
    nbox = int(lines[4].strip("(").split()[0])
    boxes = np.array([[int(v) for v in BOX.match(lines[5 + n]).groups()[:6]] for n in range(nbox)])
    assert lines[5 + nbox] == ")"
    assert int(lines[6 + nbox]) == nbox
    fod = []
    for n in range(nbox):
        tag, fname, off = lines[7 + nbox + n].split()
        assert tag == "FabOnDisk:"
        fod.append((fname, int(off)))
    k = 7 + 2 * nbox
    assert lines[k] == "" and lines[k + 1] == "%d,%d" % (nbox, ncomp)
    mins = np.array([[float(v) for v in lines[k + 2 + n].rstrip(",").split(",")] for n in range(nbox)])
    k += 2 + nbox
    assert lines[k] == "" and lines[k + 1] == "%d,%d" % (nbox, ncomp)
    maxs = np.array([[float(v) for v in lines[k + 2 + n].rstrip(",").split(",")] for n in range(nbox)])
    data = []
    d = os.path.dirname(prefix)
    for n, (fname, off) in enumerate(fod):
        with open(os.path.join(d, fname), "rb") as fh:
            fh.seek(off)
            hdr = fh.readline().decode()
            assert hdr.startswith("FAB ((8, (64 11 52 0 1 12 0 1023)),(8, (1 2 3 4 5 6 7 8)))"), hdr
            m = BOX.search(hdr[hdr.index(")))") + 3:])
            fb = [int(v) for v in m.groups()[:6]]
            nc = int(hdr.split()[-1])
            assert nc == ncomp
            shape = (ncomp, fb[5] - fb[2] + 1, fb[4] - fb[1] + 1, fb[3] - fb[0] + 1)
            data.append(np.fromfile(fh, dtype="<f8", count=int(np.prod(shape))).reshape(shape))
    return boxes, ncomp, ngrow, data, mins, maxs


def read_plotfile(path):
    """Returns a dict: names, time, finest_level, prob_lo/hi, ref_ratio,
    domains, level_steps, dx, and per level its boxes and per-box arrays
    (ncomp, nz, ny, nx)."""
    L = open(os.path.join(path, "Header")).read().split("\n")
    assert L[0] == "HyperCLaw-V1.1"
    nc = int(L[1])
    names = L[2:2 + nc]
    i = 2 + nc
    assert int(L[i]) == 3
    time = float(L[i + 1])
    finest = int(L[i + 2])
    prob_lo = [float(v) for v in L[i + 3].split()]
    prob_hi = [float(v) for v in L[i + 4].split()]
    ratio = [int(v) for v in L[i + 5].split()]
    domains = [[int(v) for v in m[:6]] for m in BOX.findall(L[i + 6])]
    steps = [int(v) for v in L[i + 7].split()]
    dx = [[float(v) for v in L[i + 8 + l].split()] for l in range(finest + 1)]
    i += 8 + finest + 1
    assert int(L[i]) == 0 and int(L[i + 1]) == 0
    i += 2
    levels = []
    for lev in range(finest + 1):
        lv, nb, t = L[i].split()
        assert int(lv) == lev
        nb = int(nb)
        lstep = int(L[i + 1])
        phys = [[float(v) for v in L[i + 2 + 3 * n + d].split()] for n in range(nb) for d in range(3)]
        rel = L[i + 2 + 3 * nb]
        boxes, ncomp, ngrow, data, mins, maxs = read_multifab(os.path.join(path, rel))
        assert ncomp == nc and ngrow == 0 and len(boxes) == nb
        levels.append({"boxes": boxes, "data": data, "phys": phys, "step": lstep, "mins": mins, "maxs": maxs,
                       "time": float(t)})
        i += 3 + 3 * nb
    return {"names": names, "time": time, "finest_level": finest, "prob_lo": prob_lo, "prob_hi": prob_hi,
            "ref_ratio": ratio, "domains": domains, "level_steps": steps, "dx": dx, "levels": levels}
