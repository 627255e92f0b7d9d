"""Queued runs into host buffers (mf_ic_run_async / mf_ic_wait): a run's
particle copies overlap the next run's fields and the next host noise upload
overlaps the run before it.  Every queued run must hand over exactly what a
synchronous mf_ic_run of the same noise hands over (bit for bit), whatever
is queued around it."""
import numpy as np
import pytest

from tests.ic_helpers import setup

pytestmark = pytest.mark.gpu
N, L, Z = 64, 100.0, 24.0


def _pipeline(ctx, prec="f32", lattice="bcc"):
    from monofonic_gb300 import ic
    cosmo, sc, osc = setup(Z)
    cfg = ic.ICConfig(ngrid=N, boxlen=L, zstart=Z, lpt_order=3, lattice=lattice, precision=prec, plt=True,
                      lunit=L, vunit=L, pos64=(prec == "f64"), id64=True)
    return ic.ICGenerator(ctx, cfg, sc)


class _HostSet:
    """page-locked host buffers for one run's particles"""

    def __init__(self, g):
        from monofonic_gb300 import ic
        self.g = g
        self.bufs = [ic.PinnedBuffer(b) for b in (g.pos_bytes, g.vel_bytes, g.id_bytes)]
        for b in self.bufs:
            b.array(np.uint8, (b.nbytes,))[...] = 0xA5  # a pattern no run writes

    @property
    def ptrs(self):
        return [b.ptr for b in self.bufs]

    def arrays(self):
        rt = np.float64 if self.g.cfg.pos64 else np.float32
        n = self.g.npart
        return (self.bufs[0].array(rt, (n, 3)).copy(), self.bufs[1].array(rt, (n, 3)).copy(),
                self.bufs[2].array(np.uint64, (n,)).copy())

    def close(self):
        for b in self.bufs:
            b.close()


def _noise(seed):
    from monofonic_gb300 import ic
    pin = ic.PinnedBuffer(N ** 3 * 8)
    pin.array(np.float64, (N, N, N))[...] = ic.white_noise(N, seed)
    return pin


def _sync(g, noise_pin, host):
    g.set_noise_host_ptr(noise_pin.ptr)
    g.run_into(*host.ptrs)
    return host.arrays()


def _same(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_queued_runs_equal_synchronous_runs(ctx, prec):
    g = _pipeline(ctx, prec)
    noises = [_noise(s) for s in (11, 12, 13)]
    ref_host = _HostSet(g)
    want = [_sync(g, nz, ref_host) for nz in noises]
    assert not _same(want[0], want[1])
    outs = [_HostSet(g) for _ in range(4)]
    order = [0, 1, 2, 0]
    for k, i in enumerate(order):
        g.set_noise_host_ptr(noises[i].ptr)
        g.run_into_async(*outs[k].ptrs)
    g.wait()
    for k, i in enumerate(order):
        assert _same(outs[k].arrays(), want[i]), (prec, k, i)
    for b in outs + [ref_host] + noises:
        b.close()
    g.close()


def test_queued_runs_into_one_buffer_set_end_with_the_last(ctx):
    """back-to-back queued runs into the same host buffers (the bench's e2e
    loop): the copies stay in run order, the buffers end with the last run"""
    g = _pipeline(ctx)
    noises = [_noise(s) for s in (21, 22)]
    ref_host = _HostSet(g)
    want_last = _sync(g, noises[1], ref_host)
    host = _HostSet(g)
    for i in (0, 1, 0, 1, 0, 1):
        g.set_noise_host_ptr(noises[i].ptr)
        g.run_into_async(*host.ptrs)
    g.wait()
    assert _same(host.arrays(), want_last)
    for b in (host, ref_host, *noises):
        b.close()
    g.close()


def test_device_run_after_queued_run(ctx):
    """a device-output run queued right after an asynchronous host run waits
    for that run's copies before it rewrites the particle buffers: the host
    set holds the first noise's particles, the device buffers the second's"""
    import ctypes as C
    import monofonic_gb300 as mf
    g = _pipeline(ctx)
    noises = [_noise(s) for s in (31, 32)]
    ref_host = _HostSet(g)
    want = [_sync(g, nz, ref_host) for nz in noises]
    host = _HostSet(g)
    g.set_noise_host_ptr(noises[0].ptr)
    g.run_into_async(*host.ptrs)
    g.set_noise_host_ptr(noises[1].ptr)
    assert mf.lib().mf_ic_enqueue(g.ptr) == 0
    g.wait()
    assert _same(host.arrays(), want[0])
    from monofonic_gb300 import _lib as Lb
    d = Lb.mf_particles()
    assert mf.lib().mf_ic_particles(g.ptr, C.byref(d)) == 0
    dev = _HostSet(g)
    for ptr, src, nb in zip(dev.ptrs, (d.pos, d.vel, d.ids), (g.pos_bytes, g.vel_bytes, g.id_bytes)):
        assert mf.lib().mf_copy_to_host(C.c_void_p(ptr), C.c_void_p(src), C.c_size_t(nb)) == 0
    assert _same(dev.arrays(), want[1])
    for b in (host, dev, ref_host, *noises):
        b.close()
    g.close()


def test_queued_run_needs_host_buffers(ctx):
    import ctypes as C
    import monofonic_gb300 as mf
    from monofonic_gb300 import _lib as Lb
    g = _pipeline(ctx)
    g.set_noise_seed(5)
    out = Lb.mf_particles()
    out.location = Lb.MF_LOC_DEVICE
    assert mf.lib().mf_ic_run_async(g.ptr, C.byref(out)) == Lb.MF_ERR_ARG
    out.location = Lb.MF_LOC_HOST  # null buffers
    assert mf.lib().mf_ic_run_async(g.ptr, C.byref(out)) == Lb.MF_ERR_ARG
    g.close()


def test_host_noise_after_stage_times_of_a_device_run(ctx):
    """a device-output run records no hand-off stage; reading the stage times
    then reports -1 for it and leaves no CUDA error behind for the next call
    (a host noise upload)"""
    import monofonic_gb300 as mf
    g = _pipeline(ctx)
    g.set_noise_seed(7)
    assert mf.lib().mf_ic_enqueue(g.ptr) == 0
    g.wait()
    assert g.stage_times()[7] == -1.0
    pin = _noise(41)
    g.set_noise_host_ptr(pin.ptr)
    host = _HostSet(g)
    g.run_into(*host.ptrs)
    pin.close()
    host.close()
    g.close()


def test_host_runs_refused_while_capturing(ctx):
    """a run into host buffers streams its copies on a second stream, so it
    is refused (MF_ERR_STATE, nothing enqueued) while the context's stream is
    being captured into a CUDA graph; the capture and the pipeline stay usable"""
    import ctypes as C
    import warnings
    import torch
    import monofonic_gb300 as mf
    from monofonic_gb300 import _lib as Lb
    g = _pipeline(ctx)
    g.set_noise_seed(3)
    host = _HostSet(g)
    out = Lb.mf_particles()
    out.pos, out.vel, out.ids = host.ptrs
    out.location = Lb.MF_LOC_HOST
    stream = torch.cuda.ExternalStream(ctx.stream(), device=torch.device("cuda", 0))
    graph = torch.cuda.CUDAGraph()
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")  # the captured graph is empty
        with torch.cuda.graph(graph, stream=stream):
            rc_async = mf.lib().mf_ic_run_async(g.ptr, C.byref(out))
            rc_sync = mf.lib().mf_ic_run(g.ptr, C.byref(out))
    assert rc_async == Lb.MF_ERR_STATE and rc_sync == Lb.MF_ERR_STATE
    g.run_into(*host.ptrs)
    pos, vel, ids = host.arrays()
    assert np.all(np.isfinite(pos)) and ids[0] == 0
    host.close()
    g.close()
