"""Host side of the Python server wrapper without a GPU: the output callback
assembles a request's particles from the chunks the server streams
(include/monofonic_gb300_batch.h mf_output_fn), for every position / ID
width, in any chunking."""
import ctypes as C
import threading

import numpy as np
import pytest

from monofonic_gb300 import _lib as L
from monofonic_gb300.serve import Request, Server


def _server(output):
    s = Server.__new__(Server)  # the callback only, no device server behind it
    s.output, s.results, s.bytes_out, s._lock, s._reqs = output, {}, 0, threading.Lock(), {}
    s.ptr = None
    return s


@pytest.mark.parametrize("pos64,id64", [(True, True), (False, True), (False, False)])
@pytest.mark.parametrize("chunk", [1000, 4096, 5000])
def test_chunks_assemble_the_request(pos64, id64, chunk):
    req = Request(ngrid=16, boxlen=32.0, lattice="bcc", pos64=pos64, id64=id64)
    n = req.npart
    rt, it = (np.float64 if pos64 else np.float32), (np.uint64 if id64 else np.uint32)
    rng = np.random.default_rng(chunk)
    pos, vel = rng.standard_normal((n, 3)).astype(rt), rng.standard_normal((n, 3)).astype(rt)
    ids = rng.permutation(n).astype(it)
    s = _server("collect")
    rid = 7
    s._reqs[rid] = req
    s.results[rid] = (np.empty((n, 3), rt), np.empty((n, 3), rt), np.empty(n, it))
    for first in range(0, n, chunk):
        cnt = min(chunk, n - first)
        # one staging buffer holding the chunk's positions, velocities and IDs back to back
        stage = np.concatenate([pos[first:first + cnt].view(np.uint8).ravel(), vel[first:first + cnt].view(np.uint8).ravel(),
                                ids[first:first + cnt].view(np.uint8).ravel()])
        part = L.mf_particles()
        base = stage.ctypes.data
        part.pos, part.vel = base, base + pos[:cnt].nbytes
        part.ids = base + 2 * pos[:cnt].nbytes
        part.npart, part.location = cnt, L.MF_LOC_HOST
        s._on_chunk(None, rid, C.pointer(part), first, cnt, int(first + cnt == n))
    got = s.results[rid]
    assert np.array_equal(got[0], pos) and np.array_equal(got[1], vel) and np.array_equal(got[2], ids)
    assert s.bytes_out == n * (6 * (8 if pos64 else 4) + (8 if id64 else 4))


def test_count_mode_only_counts():
    req = Request(ngrid=16, boxlen=32.0)
    s = _server("count")
    s._reqs[3] = req
    part = L.mf_particles()
    s._on_chunk(None, 3, C.pointer(part), 0, 100, 0)
    assert s.bytes_out == 100 * 56 and 3 not in s.results
