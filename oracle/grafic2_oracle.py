"""GRAFIC-2 / RAMSES output format in numpy (test infrastructure only).

This module is the checker, never the product: only ``tests/`` may import it.
It restates the bytes that src/plugins/output_grafic2.cc writes (header
record, one Fortran record per plane, file names, the components the plugin
skips, the ramses.nml namelist), each function citing the lines it follows
(paths relative to the monofonIC source tree).

Parity status: the reference ships no GRAFIC-2 files, fixtures or tests, and
cannot be built here, so this restatement is pinned only to the plugin's
source as read; the namelist text is additionally checked against a literal
copy of the expected output in the tests.
"""
from __future__ import annotations

import os

import numpy as np

# output_grafic2.cc:38-43
HEADER_DTYPE = np.dtype([("n1", "<i4"), ("n2", "<i4"), ("n3", "<i4"), ("dxini0", "<f4"), ("xoff10", "<f4"),
                         ("xoff20", "<f4"), ("xoff30", "<f4"), ("astart0", "<f4"), ("omega_m0", "<f4"),
                         ("omega_l0", "<f4"), ("h00", "<f4")])

SPECIES_LETTER = {"dm": "c", "baryon": "b", "neutrino": "n"}


def header(ngrid, boxlen, zstart, H0, Omega_m, Omega_DE):
    """header_ of the constructor (output_grafic2.cc:66-99): double
    expressions rounded to the float fields"""
    h = np.zeros((), dtype=HEADER_DTYPE)
    h["n1"] = h["n2"] = h["n3"] = ngrid
    h["dxini0"] = np.float32(boxlen / (H0 * 0.01) / ngrid)
    h["astart0"] = np.float32(1.0 / (1.0 + zstart))
    h["omega_m0"] = np.float32(Omega_m)
    h["omega_l0"] = np.float32(Omega_DE)
    h["h00"] = np.float32(H0)
    return h


def _record(payload: bytes) -> bytes:
    m = np.uint32(len(payload)).tobytes()
    return m + payload + m


def file_bytes(field, hdr) -> bytes:
    """write_grid_data (output_grafic2.cc:186-236): header record, then for
    each plane i of the grid's third index the record of
    data_buf_[j*ngrid + k] = g(k, j, i) as float"""
    f = np.asarray(field)
    n = f.shape[0]
    parts = [_record(hdr.tobytes())]
    for i in range(n):
        plane = np.ascontiguousarray(f[:, :, i].T).astype(np.float32)  # [j][k] = g(k, j, i)
        parts.append(_record(plane.tobytes()))
    return b"".join(parts)


def file_name(dirname, species, component):
    """get_file_name (output_grafic2.cc:139-184)"""
    s = SPECIES_LETTER[species]
    base = {"density": "delta" + s, "vx": "vel" + s + "x", "vy": "vel" + s + "y", "vz": "vel" + s + "z",
            "dx": "pos" + s + "x", "dy": "pos" + s + "y", "dz": "pos" + s + "z", "mass": "mass" + s}[component]
    return os.path.join(dirname, "ic_" + base)


def ignores(species, component):
    """components write_grid_data returns on (output_grafic2.cc:189-193)"""
    if species == "dm" and component == "density":
        return True
    return species == "baryon" and component in ("dx", "dy", "dz", "mass")


def ramses_namelist(dirname, ngrid, Omega_b, baryons=False):
    """write_ramses_namelist (output_grafic2.cc:249-320); the double omega_b
    is streamed with the default ostream format, i.e. printf's %g"""
    levelmin = int(round(np.log2(ngrid)))
    naddref = 5
    return ("&RUN_PARAMS\ncosmo=.true.\npic=.true.\npoisson=.true.\n"
            + ("hydro=.true.\n" if baryons else "hydro=.false.\n")
            + "nrestart=0\nnremap=1\nnsubcycle=1,2\nncontrol=1\nverbose=.false.\n/\n\n"
            + "&INIT_PARAMS\nfiletype='grafic'\n" + ("omega_b=%g\n" % Omega_b)
            + "initfile(1)='" + dirname + "'\n/\n\n"
            + "&AMR_PARAMS\nlevelmin=%d\nlevelmax=%d\nnexpand=1" % (levelmin, levelmin + naddref)
            + "\nngridmax=2000000\nnpartmax=3000000\n/\n\n"
            + "&REFINE_PARAMS\nm_refine=%d*8.,\n/\n" % (1 + naddref))


def read(path):
    """parse a GRAFIC-2 file: (header, float32 field f[i][j][k]) with every
    record marker checked"""
    raw = np.fromfile(path, dtype=np.uint8)
    pos = 0

    def rec():
        nonlocal pos
        m0 = int(raw[pos:pos + 4].view("<u4")[0])
        body = raw[pos + 4:pos + 4 + m0]
        m1 = int(raw[pos + 4 + m0:pos + 8 + m0].view("<u4")[0])
        assert m0 == m1, "record markers differ"
        pos += 8 + m0
        return body

    h = rec().view(HEADER_DTYPE)[0]
    n1, n2, n3 = int(h["n1"]), int(h["n2"]), int(h["n3"])
    f = np.empty((n1, n2, n3), dtype=np.float32)
    for i in range(n3):
        plane = rec().view("<f4").reshape(n2, n1)  # [j][k]
        f[:, :, i] = plane.T
    assert pos == raw.size, "trailing bytes"
    return h, f
