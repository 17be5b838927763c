"""Writers of small synthetic AMRVAC data files, in the layouts the reference's
reader parses (fomo-c/example/example_mpi_amrvac/read_amrvac_files.cpp), for
the AMRVAC ingestion tests.  TEST INFRASTRUCTURE.

* ``write_new``: a version 3 or 4 data file (header with the domain, tree at
  ``treeoffset``, leaf blocks at ``blockoffset``, two ghost-cell counts per
  dimension before each block; :430-528, :535-683).  The header length is not
  a multiple of 8, so the blocks' doubles start unaligned in the file.
* ``write_old``: a pre-2017 data file (blocks first, then the tree, the block
  size, the equation parameters and the trailer; :301-418) and its amrvac.par
  file (nxlone, xprobmin, xprobmax; :50-112).

Level-1 blocks listed in ``refine`` are refined once: the tree holds a parent
flag (0) followed by its 2^ndim children (leaves, 1).  The MHD variables
(rho, m1, m2, m3, e, b1, b2, b3) are seeded random fields with rho > 0 and a
positive pressure.  The same arguments give the same bytes on every machine.
"""

from __future__ import annotations

import struct

import numpy as np

NW = 8
GAMMA = 5.0 / 3.0


def _morton(i: int, j: int, k: int) -> int:
    r = 0
    for b in range(21):
        r |= ((i >> b) & 1) << (3 * b) | ((j >> b) & 1) << (3 * b + 1) | ((k >> b) & 1) << (3 * b + 2)
    return r


def _tree(nblocks, refine, ndim, order):
    """Forest flags and leaves (level, 1-based index) in the reader's walk order."""
    nb = list(nblocks) + [1] * (3 - ndim)
    top = [(i, j, k) for k in range(nb[2]) for j in range(nb[1]) for i in range(nb[0])]
    if order == "morton":
        top.sort(key=lambda t: _morton(*t))
    forest, leaves = [], []
    for (i, j, k) in top:
        key = (i, j, k)[:ndim]
        if key in refine:
            forest.append(0)
            for c in range(1 << ndim):
                ni = 2 * i + 1 + c % 2
                if ndim == 2:
                    nj, nk = 2 * j + 1 + c // 2, 1
                else:
                    nj, nk = 2 * j + 1 + (c // 2) % 2, 2 * k + 1 + c // 4
                forest.append(1)
                leaves.append((2, ni, nj, nk))
        else:
            forest.append(1)
            leaves.append((1, i + 1, j + 1, k + 1))
    return forest, leaves


def _blocks(nleafs, nglev1, seed):
    """nleafs blocks of the 8 MHD variables, each variable-major (nw x nglev1)."""
    rng = np.random.default_rng(seed)
    rho = 1.0 + 0.5 * rng.random((nleafs, nglev1))
    v = rng.uniform(-0.3, 0.3, (3, nleafs, nglev1))
    b = rng.uniform(-0.2, 0.2, (3, nleafs, nglev1))
    p = 0.1 + 0.2 * rng.random((nleafs, nglev1))
    e = p / (GAMMA - 1.0) + 0.5 * rho * (v ** 2).sum(0) + 0.5 * (b ** 2).sum(0)
    out = np.stack([rho, rho * v[0], rho * v[1], rho * v[2], e, b[0], b[1], b[2]], axis=1)  # leaf, var, cell
    return np.ascontiguousarray(out, dtype="<f8")


def _name(s: str, pad: bytes) -> bytes:
    return s.encode().ljust(16, pad)


def write_new(path, version=4, ndim=3, nblocks=(2, 2, 2), nx=(4, 4, 4), refine=((1, 0, 1),),
              xprobmin=(-5.0, -5.0, -5.0), xprobmax=(5.0, 5.0, 5.0), seed=1, pad=b"\0"):
    nblocks, nx = tuple(nblocks[:ndim]), tuple(nx[:ndim])
    refine = {tuple(r[:ndim]) for r in refine}
    forest, leaves = _tree(nblocks, refine, ndim, "morton")
    nleafs, nparents = len(leaves), len(refine)
    nglev1 = int(np.prod(nx))
    data = _blocks(nleafs, nglev1, seed)
    hdr = struct.pack("<10i", version, 0, 0, NW, 3, ndim, 2 if refine else 1, nleafs, nparents, 0)
    hdr += struct.pack("<d", 0.0)
    hdr += struct.pack(f"<{ndim}d", *xprobmin[:ndim]) + struct.pack(f"<{ndim}d", *xprobmax[:ndim])
    hdr += struct.pack(f"<{ndim}i", *[nb * n for nb, n in zip(nblocks, nx)]) + struct.pack(f"<{ndim}i", *nx)
    hdr += b"".join(_name(s, pad) for s in ("rho", "m1", "m2", "m3", "e", "b1", "b2", "b3")) + _name("mhd", pad)
    hdr += struct.pack("<i", 1) + struct.pack("<d", GAMMA) + _name("gamma", pad)
    treeoff = len(hdr)
    tree = struct.pack(f"<{len(forest)}i", *forest)
    blockoff = treeoff + len(tree)
    hdr = hdr[:4] + struct.pack("<2i", treeoff, blockoff) + hdr[12:]
    body = b"".join(struct.pack(f"<{2 * ndim}i", *([0] * (2 * ndim))) + data[b].tobytes() for b in range(nleafs))
    with open(path, "wb") as f:
        f.write(hdr + tree + body)
    return nleafs * nglev1


def write_old(path, par_path, order="gitlab", ndim=3, nblocks=(2, 2, 2), nx=(4, 4, 4), refine=((0, 1, 1),),
              xprobmin=(-4.0, -6.0, -2.0), xprobmax=(4.0, 2.0, 6.0), seed=2):
    nblocks, nx = tuple(nblocks[:ndim]), tuple(nx[:ndim])
    refine = {tuple(r[:ndim]) for r in refine}
    forest, leaves = _tree(nblocks, refine, ndim, "morton" if order == "gitlab" else "xfast")
    nleafs = len(leaves)
    nglev1 = int(np.prod(nx))
    data = _blocks(nleafs, nglev1, seed)
    eqpar = (0.0, GAMMA)  # gamma_eqparposition = 1
    out = data.tobytes() + struct.pack(f"<{len(forest)}i", *forest) + struct.pack(f"<{ndim}i", *nx)
    out += struct.pack(f"<{len(eqpar)}d", *eqpar)
    out += struct.pack("<7i", nleafs, 2 if refine else 1, ndim, 3, NW, len(eqpar), 0) + struct.pack("<d", 0.0)
    with open(path, "wb") as f:
        f.write(out)
    lines = [" &meshlist"]
    for d in range(ndim):
        lines.append(f"        nxlone{d + 1}={nblocks[d] * nx[d]}")
    for d in range(ndim):
        lines.append(f"        xprobmin{d + 1}={xprobmin[d]!r}")
        lines.append(f"        xprobmax{d + 1}= {xprobmax[d]!r}")
    lines.append(" /")
    with open(par_path, "w") as f:
        f.write("\n".join(lines) + "\n")
    return nleafs * nglev1


# The golden cases: name -> (writer, arguments, reader arguments)
CASES = {
    "v4_3d": ("new", dict(version=4, ndim=3), dict(amrvac_version="gitlab", gamma_eqparposition=0)),
    "v4_2d": ("new", dict(version=4, ndim=2, nblocks=(4, 4), nx=(4, 4), refine=((2, 1),),
                          xprobmin=(-3.0, -1.0), xprobmax=(5.0, 7.0), seed=3),
              dict(amrvac_version="gitlab", gamma_eqparposition=0)),
    "old_3d_gitlab": ("old", dict(order="gitlab", ndim=3), dict(amrvac_version="gitlab", gamma_eqparposition=1)),
    "old_2d_xfast": ("old", dict(order="old", ndim=2, nblocks=(4, 2), nx=(4, 4), refine=((3, 0),),
                                 xprobmin=(0.0, -2.0), xprobmax=(16.0, 6.0), seed=4),
                     dict(amrvac_version="old", gamma_eqparposition=1)),
}
UNITS = dict(n_unit=1e9, Teunit=1e6, L_unit=2.0)


def write_case(name, directory):
    """Write golden case `name` into `directory`; returns (datfile, parfile or None, reader kwargs)."""
    import os
    kind, args, rargs = CASES[name]
    dat = os.path.join(directory, name + ".dat")
    par = None
    if kind == "new":
        write_new(dat, **args)
    else:
        par = os.path.join(directory, name + ".par")
        write_old(dat, par, **args)
    return dat, par, dict(rargs, **UNITS)
