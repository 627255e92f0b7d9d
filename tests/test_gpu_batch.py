"""Device white noise, replayable pipelines, the recorded batch and the
continuous-batching server.  Every realization is deterministic, so a
realization made in a batch or in a mixed server load is bit-identical to the
same request run alone."""
import os

import numpy as np
import pytest

from oracle import lpt_oracle as O
from tests.ic_helpers import lattice_q, rel_l2

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _standalone(ctx, req):
    """the request through the single-pipeline API (ICGenerator)"""
    from monofonic_gb300 import ic
    sc = ic.cosmology_scalars(req.cosmology, req.zstart)
    cfg = ic.ICConfig(ngrid=req.ngrid, boxlen=req.boxlen, zstart=req.zstart, lpt_order=req.lpt_order,
                      lattice=req.lattice, precision=req.precision, lunit=req.boxlen, vunit=req.boxlen,
                      pos64=req.pos64, id64=req.id64)
    g = ic.ICGenerator(ctx, cfg, sc)
    g.set_noise_seed(req.seed)
    out = g.run()
    g.close()
    return out


def _same(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_device_noise_is_bit_identical_to_host(ctx, prec):
    import monofonic_gb300 as mf
    from monofonic_gb300 import ic
    for n, seed in ((16, 12345), (32, 77), (64, 2 ** 40 + 5)):
        g = mf.Grid_FFT(ctx, n, 1.0, prec)
        g.fill_white_noise(seed)
        got = g.get_real()
        ref = ic.white_noise(n, seed)
        if prec == "f64":
            assert np.array_equal(got, ref)
        else:
            assert np.array_equal(got, ref.astype(np.float32))
    fx = np.load(os.path.join(ROOT, "tests", "golden", "noise_n16_seed12345.npy"))
    g = mf.Grid_FFT(ctx, 16, 1.0, "f64")
    g.fill_white_noise(12345)
    assert np.array_equal(g.get_real(), fx)


def test_seeded_pipeline_equals_uploaded_noise(ctx):
    """device noise from a seed = the host plugin's field uploaded; FP64
    plain against the oracle on that field"""
    from monofonic_gb300 import ic
    from monofonic_gb300.serve import Request
    from tests.ic_helpers import setup
    cosmo, sc, osc = setup(24.0)
    req = Request(ngrid=32, boxlen=64.0, zstart=24.0, lpt_order=3, lattice="bcc", precision="f64",
                  cosmology=cosmo, seed=4711)
    a = _standalone(ctx, req)
    cfg = ic.ICConfig(ngrid=32, boxlen=64.0, zstart=24.0, lpt_order=3, lattice="bcc", precision="f64",
                      lunit=64.0, vunit=64.0)
    g = ic.ICGenerator(ctx, cfg, sc)
    noise = ic.white_noise(32, 4711)
    g.set_noise(noise)
    assert _same(a, g.run())
    f = O.lpt_potentials(noise, 64.0, 3, osc)
    rpos, rvel, rids = O.particles(f, 64.0, 3, osc.vfac, lattice=1, lunit=64.0, vunit=64.0)
    q = lattice_q(32, 1, 64.0)
    assert rel_l2(a[0] - q, rpos - q) < 1e-12
    assert rel_l2(a[1], rvel) < 1e-12
    assert np.array_equal(a[2], rids)


def test_set_cosmology_equals_fresh_pipeline(ctx):
    from monofonic_gb300 import ic
    from monofonic_gb300.serve import Request
    c1 = ic.Cosmology(Omega_m=0.27, sigma_8=0.75, n_s=0.93)
    c2 = ic.Cosmology(Omega_m=0.33, sigma_8=0.88, n_s=0.99)
    r1 = Request(ngrid=32, boxlen=64.0, lpt_order=3, precision="f32", cosmology=c1, seed=5)
    r2 = Request(ngrid=32, boxlen=64.0, lpt_order=3, precision="f32", cosmology=c2, seed=6)
    cfg = ic.ICConfig(ngrid=32, boxlen=64.0, zstart=24.0, lpt_order=3, precision="f32", lunit=64.0, vunit=64.0)
    g = ic.ICGenerator(ctx, cfg, ic.cosmology_scalars(c1, 24.0))
    g.set_noise_seed(5)
    a1 = g.run()
    g.set_cosmology(ic.cosmology_scalars(c2, 24.0))
    g.set_noise_seed(6)
    a2 = g.run()
    assert _same(a1, _standalone(ctx, r1))
    assert _same(a2, _standalone(ctx, r2))
    assert not np.array_equal(a1[0], a2[0])


def _mixed_requests(rng, n_items, sizes, prec="f32"):
    from monofonic_gb300 import ic
    from monofonic_gb300.serve import Request
    out = []
    for i in range(n_items):
        n = int(rng.choice(sizes))
        c = ic.Cosmology(Omega_m=float(rng.uniform(0.25, 0.35)), sigma_8=float(rng.uniform(0.7, 0.9)),
                         n_s=float(rng.uniform(0.92, 1.0)))
        out.append(Request(ngrid=n, boxlen=2.0 * n, zstart=24.0, lpt_order=int(rng.choice([2, 3])),
                           precision=prec, cosmology=c, seed=int(rng.integers(1, 2 ** 62))))
    return out


def test_batch_equals_standalone_and_replays(ctx):
    from monofonic_gb300.serve import Batch
    rng = np.random.default_rng(11)
    reqs = _mixed_requests(rng, 7, [16, 32, 64])
    reqs[3].precision = "f64"
    reqs[5].lattice = "bcc"
    b = Batch(reqs, nstreams=3, autotune=True)
    assert "conv_z" in b.tuning
    info = b.info()
    assert info["graph_nodes"] > info["kernels"] > 0
    ms = b.run()
    assert ms > 0
    for i, r in enumerate(reqs):
        assert _same(b.particles(i), _standalone(ctx, r)), i
    # replay the same graph with new seeds and cosmologies
    new = _mixed_requests(np.random.default_rng(12), 7, [16])
    b.set_items(0, cosmologies=[r.cosmology for r in new], seeds=[r.seed for r in new])
    b.run()
    for i, r in enumerate(b.requests):
        assert _same(b.particles(i), _standalone(ctx, r)), i
    b.close()


def test_server_result_alone_equals_result_in_mix(ctx):
    from monofonic_gb300.serve import Server
    rng = np.random.default_rng(3)
    reqs = _mixed_requests(rng, 10, [16, 32, 64])
    reqs[4].precision = "f64"
    probe = reqs[6]
    alone = Server(nworkers=1, output="collect", chunk_particles=5000)
    rid = alone.submit(probe)
    res = alone.wait(rid, 120.0)
    assert res["status"] == 0
    ref = alone.results[rid]
    alone.close()
    mix = Server(nworkers=4, output="collect", chunk_particles=7000)
    ids = [mix.submit(r) for r in reqs]
    mix.drain(300.0)
    st = mix.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert _same(mix.results[ids[6]], ref)
    for i in (0, 4, 9):
        assert _same(mix.results[ids[i]], _standalone(ctx, reqs[i])), i
    # requests overlapped on the device: some were admitted before others finished
    rs = [mix.wait(i) for i in ids]
    assert any(a["t_admit"] < b["t_gpu_done"] and b["t_admit"] < a["t_gpu_done"]
               for a in rs for b in rs if a["id"] < b["id"])
    mix.close()


def test_server_admission_respects_budget(ctx):
    from monofonic_gb300 import ic
    from monofonic_gb300.serve import Server, Request
    reqs = [Request(ngrid=n, boxlen=2.0 * n, lpt_order=o, precision="f32", seed=s)
            for s, (n, o) in enumerate([(64, 3), (32, 2), (64, 2), (32, 3), (64, 3), (16, 3)])]
    sizes = []
    for r in reqs:
        cfg = ic.ICConfig(ngrid=r.ngrid, boxlen=r.boxlen, zstart=r.zstart, lpt_order=r.lpt_order,
                          precision=r.precision, lunit=r.boxlen, vunit=r.boxlen)
        sizes.append(ic.device_footprint(cfg, ic.cosmology_scalars(r.cosmology, r.zstart)))
    budget = int(max(sizes) * 1.2)  # room for one large pipeline at a time
    srv = Server(nworkers=3, hbm_budget=budget, output=None)
    ids = [srv.submit(r) for r in reqs]
    srv.drain(300.0)
    st = srv.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["peak_bytes"] <= budget
    with pytest.raises(Exception):
        srv.submit(Request(ngrid=256, boxlen=512.0, lpt_order=3))  # larger than the budget
    srv.close()


def test_server_poll_and_cancel(ctx):
    """one worker: the first request is still creating its pipeline when the
    last ones are cancelled, so they leave the queue without running; the
    others finish normally and cancelling a finished request is an error"""
    from monofonic_gb300 import _lib as L
    from monofonic_gb300.serve import Server, Request
    srv = Server(nworkers=1, output="count")
    reqs = [Request(ngrid=128, boxlen=256.0, lpt_order=3, seed=1), Request(ngrid=32, boxlen=64.0, seed=2),
            Request(ngrid=64, boxlen=128.0, seed=3), Request(ngrid=64, boxlen=128.0, seed=4)]
    ids = [srv.submit(r) for r in reqs]
    srv.cancel(ids[2])
    srv.cancel(ids[3])
    for i in (2, 3):  # finished at once, never admitted
        res = srv.poll(ids[i])
        assert res is not None and res["status"] == L.MF_ERR_CANCELLED and res["t_admit"] == 0.0
    srv.drain(300.0)
    for i in (0, 1):
        res = srv.poll(ids[i])
        assert res is not None and res["status"] == 0 and res["npart"] == reqs[i].npart
        assert res == srv.wait(ids[i])
    st = srv.stats()
    assert st["completed"] == 2 and st["failed"] == 2 and st["queued"] == 0
    assert srv.bytes_out == sum(r.npart * 56 for r in reqs[:2])  # FP64 positions and velocities, u64 IDs
    with pytest.raises(L.MFError) as e:
        srv.cancel(ids[0])
    assert e.value.code == L.MF_ERR_STATE
    with pytest.raises(L.MFError):
        srv.poll(len(ids))
    # released records answer MF_ERR_STATE; the others stay readable
    srv.release(ids[0])
    srv.release(ids[2])
    for call in (srv.poll, srv.wait, srv.release, srv.cancel):
        with pytest.raises(L.MFError) as e:
            call(ids[0])
        assert e.value.code == L.MF_ERR_STATE
    assert srv.poll(ids[1])["status"] == 0 and srv.stats()["completed"] == 2
    srv.drain(10.0)
    srv.close()


def test_autotune_keeps_parity(ctx):
    """the autotuner changes schedules only: a convolution after tuning still
    matches the oracle (FP64 1e-12), and the report names every pass"""
    import monofonic_gb300 as mf
    from monofonic_gb300 import ic
    n, L = 32, 100.0
    rep = ic.autotune(ctx, n, "f64")
    for k in ("conv_xinv", "conv_yinv", "conv_z", "conv_yfwd", "conv_xfwd"):
        assert f"{k} L=48 f64" in rep, rep
    rng = np.random.default_rng(5)
    x = rng.standard_normal((n, n, n))
    g = mf.Grid_FFT(ctx, n, L, "f64")
    g.set_real(x)
    g.FourierTransformForward()
    out = mf.Grid_FFT(ctx, n, L, "f64", "k")
    cv = mf.OrszagConvolver(ctx, n, L, "f64")
    cv.convolve_Hessians(g, (0, 1), g, (2, 2), mf.op.assign_to(out))
    phi = O.r2c(x)
    ref = O.orszag_conv2(O.hessian(phi, L, 0, 1), O.hessian(phi, L, 2, 2))
    assert rel_l2(out.get_k(), ref) < 1e-12
    ic.autotune_reset()


@pytest.mark.parametrize("prec,tol", [("f64", 1e-12), ("f32", 1e-5)])
def test_every_schedule_candidate_keeps_parity(ctx, prec, tol):
    """each schedule the autotuner may pick, forced by hand: 1 or 2 CTAs per SM
    for every pass, and the direct-load radix-4 z pass"""
    import monofonic_gb300 as mf
    from monofonic_gb300 import ic
    lib = mf.lib()
    pc = 0 if prec == "f64" else 1
    L = 100.0
    for n in (16, 32, 64):
        M = 3 * n // 2
        rng = np.random.default_rng(n)
        x = rng.standard_normal((n, n, n))
        phi = O.r2c(x)
        ref = O.orszag_conv2(O.hessian(phi, L, 0, 0), O.sum_hessian(phi, L, (1, 1), (2, 2)))
        g = mf.Grid_FFT(ctx, n, L, prec)
        g.set_real(x)
        g.FourierTransformForward()
        cv = mf.OrszagConvolver(ctx, n, L, prec)
        for occ, zvar in ((1, 0), (2, 0), (0, 1), (1, 1)):
            for kind in range(5):
                assert lib.mf_schedule_set(kind, M, pc, occ, zvar if kind == 2 else 0) == 0
            out = mf.Grid_FFT(ctx, n, L, prec, "k")
            cv.convolve_SumOfHessians(g, (0, 0), g, (1, 1), (2, 2), mf.op.assign_to(out))
            assert rel_l2(out.get_k(), ref) < tol, (n, occ, zvar)
        ic.autotune_reset()
