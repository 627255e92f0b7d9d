"""Initial conditions pinned to the reference itself.

Each case is a monofonIC configuration (the reference's own [setup] /
[cosmology] / [random] / [output] keys) run three ways:
  * by oracle/_ref, the reference's unmodified sources compiled against the
    project shims (oracle/refrun.py), here in the build container;
  * by the numpy oracle (oracle/lpt_oracle.py), in the CPU tests;
  * by the CUDA pipeline through the C ABI, in the GPU tests, against the
    fixtures tests/golden/make_ref_fixtures.py wrote from oracle/_ref runs.
The white noise is the project RNG plugin's (the same bits on every side) and
the cosmology scalars are the ones the reference computed (stored in each
fixture).  Small cases are stored whole; large ones as a fixed random sample
of particles / cells plus exact sums of squares over all of them.
"""
from __future__ import annotations

import json
import math
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
LAT = {"sc": 0, "bcc": 1, "fcc": 2, "rsc": 3}
COSMO = dict(Omega_m=0.3099, Omega_b=0.0488, h=0.6774, sigma_8=0.8102, n_s=0.9667)

CASES = {
    # 3LPT on a body-centred lattice (2 x 16^3 particles)
    "lpt3_bcc_n16": dict(ngrid=16, boxlen=40.0, zstart=24.0, lpt_order=3, lattice="bcc", seed=777),
    # the same with the PLT corrections (particle_plt.hh, 64^3 eigen tables)
    "lpt3_bcc_plt_n16": dict(ngrid=16, boxlen=40.0, zstart=24.0, lpt_order=3, lattice="bcc", seed=777, plt=True),
    # aliased convolver, mode fixing and phase inversion
    "lpt2_sc_naive_fixinv_n16": dict(ngrid=16, boxlen=40.0, zstart=24.0, lpt_order=2, lattice="sc", seed=11,
                                     convolver="naive", fixing=True, inversion=True),
    # first order on a larger grid
    "lpt1_sc_n32": dict(ngrid=32, boxlen=64.0, zstart=49.0, lpt_order=1, lattice="sc", seed=5),
    # multi-shift lattices (chained relative shift_field readouts)
    "lpt3_fcc_n16": dict(ngrid=16, boxlen=40.0, zstart=30.0, lpt_order=3, lattice="fcc", seed=31),
    "lpt3_rsc_n16": dict(ngrid=16, boxlen=40.0, zstart=30.0, lpt_order=3, lattice="rsc", seed=31),
    # two species: dark matter and baryon particles with masses
    "baryons_lpt2_bcc_n16": dict(ngrid=16, boxlen=40.0, zstart=24.0, lpt_order=2, lattice="bcc", seed=13,
                                 baryons=True),
    # field output: dark-matter Lagrangian fields and mass field, baryons
    # through the semiclassical (PPT) Eulerian branch
    "fields_baryons_eulerian_lpt2_sc_n16": dict(ngrid=16, boxlen=40.0, zstart=24.0, lpt_order=2, lattice="sc",
                                                seed=17, baryons=True, out="field_lagrangian",
                                                baryon_out="field_eulerian"),
    # configuration 1: 2LPT, N = 64, SC, L = 100, z = 49, float64 field output
    "config1_lpt2_sc_n64_fields": dict(ngrid=64, boxlen=100.0, zstart=49.0, lpt_order=2, lattice="sc", seed=12345,
                                       out="field_lagrangian", threads=8),
    # configuration 2: 3LPT, N = 256, SC, L = 500, z = 24
    "config2_lpt3_sc_n256": dict(ngrid=256, boxlen=500.0, zstart=24.0, lpt_order=3, lattice="sc", seed=12345,
                                 threads=8),
    # configuration 3 at N = 256 (same box per cell, L = 500): 3LPT + PLT, BCC
    "config3_lpt3_bcc_plt_n256": dict(ngrid=256, boxlen=500.0, zstart=24.0, lpt_order=3, lattice="bcc",
                                      plt=True, seed=12345, threads=8),
}

FULL_LIMIT = 8192  # particles or cells stored whole up to this count
NSAMPLE = 2048


def fixture_path(name):
    return os.path.join(GOLDEN, f"ref_{name}.npz")


def lattice_q(n, lattice, unit=1.0):
    """unperturbed lattice positions in particle order (particle_generator.hh:47-63,524-541)."""
    from oracle import lpt_oracle as O
    idx = np.arange(n, dtype=np.float64)
    out = []
    for s in O.LATTICE_SHIFTS[LAT[lattice] if isinstance(lattice, str) else lattice]:
        q = np.stack(np.meshgrid((idx + s[0]) / n, (idx + s[1]) / n, (idx + s[2]) / n, indexing="ij"), -1)
        out.append(q.reshape(-1, 3) * unit)
    return np.concatenate(out)


def _fsum2(a):
    a = np.asarray(a, dtype=np.float64).reshape(-1)
    return math.fsum((a * a).tolist())


def _sample_idx(count, seed=0):
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(count, size=min(NSAMPLE, count), replace=False))


def to_fixture_keys(case: dict, res: dict) -> dict:
    """outputs keyed as the reference's capture plugin names them, particle
    positions turned into displacements from the unperturbed (primary or, for
    baryons, secondary) lattice; entries that are not arrays are dropped"""
    n, L = case["ngrid"], case["boxlen"]
    out = {}
    for key, arr in res.items():
        if not isinstance(arr, np.ndarray) or key.startswith("_") or key == "pk":
            continue
        a = np.asarray(arr)
        if key.endswith("_pos"):
            sp = key[:-4]
            q = lattice_q(n, case["lattice"], L)
            if sp == "baryon":
                q = q + _baryon_shift(case) * L
            a = a.astype(np.float64) - q
            key = sp + "_disp"
        out[key] = a
    return out


def reduce_outputs(case: dict, res: dict) -> dict:
    """what a fixture stores of one run's outputs: whole arrays for small
    runs, else a fixed sample of rows (particles) or cells (fields) plus the
    exact sum of squares over the whole array"""
    out = {}
    for key, a in to_fixture_keys(case, res).items():
        if key.endswith("_pk"):
            out[key] = a
            continue
        rows = a.shape[0] if a.ndim <= 2 else a.size
        if rows <= FULL_LIMIT:
            out[key] = a
        else:
            flat = a.reshape(a.shape[0], -1) if a.ndim <= 2 else a.reshape(-1)
            idx = _sample_idx(flat.shape[0])
            out[key + "@idx"] = idx
            out[key + "@sample"] = flat[idx]
            if a.dtype.kind == "f":
                out[key + "@sumsq"] = np.array(_fsum2(a))
    return out


def _baryon_shift(case):
    """the secondary lattice shift in box units (particle_generator.hh:56-63)"""
    from oracle import lpt_oracle as O
    return np.asarray(O.SECOND_LATTICE_SHIFT[LAT[case["lattice"]]]) / case["ngrid"]


def load_fixture(name):
    z = np.load(fixture_path(name), allow_pickle=False)
    case = json.loads(str(z["case"]))
    scalars = json.loads(str(z["scalars"]))
    arrays = {k: z[k] for k in z.files if k not in ("case", "scalars")}
    return case, scalars, arrays


def compare(got: dict, want: dict, tol_real: float, what: str = ""):
    """got: full arrays keyed as the fixture (positions already as
    displacements); want: the fixture's arrays.  Returns a list of
    (key, rel error) and raises AssertionError beyond tol_real; integer
    arrays must match exactly."""
    report = []
    keys = sorted({k.split("@")[0] for k in want})
    for key in keys:
        g = np.asarray(got[key])
        if key in want:
            w = want[key]
            if w.dtype.kind in "ui":
                assert np.array_equal(g.astype(w.dtype), w), f"{what} {key}: integer arrays differ"
                report.append((key, 0.0))
                continue
            err = float(np.linalg.norm(g - w) / max(np.linalg.norm(w), 1e-300))
            report.append((key, err))
            assert err < tol_real, f"{what} {key}: rel-L2 {err:.3e} > {tol_real:.0e}"
            continue
        idx = want[key + "@idx"]
        flat = g.reshape(g.shape[0], -1) if g.ndim <= 2 else g.reshape(-1)
        s = flat[idx]
        w = want[key + "@sample"]
        if w.dtype.kind in "ui":
            assert np.array_equal(s.astype(w.dtype), w), f"{what} {key}: integer sample differs"
            report.append((key, 0.0))
            continue
        err = float(np.linalg.norm(s - w) / max(np.linalg.norm(w), 1e-300))
        report.append((key + "@sample", err))
        assert err < tol_real, f"{what} {key} sample: rel-L2 {err:.3e} > {tol_real:.0e}"
        if key + "@sumsq" in want:
            ss = _fsum2(g)
            e2 = abs(ss - float(want[key + "@sumsq"])) / float(want[key + "@sumsq"])
            report.append((key + "@sumsq", e2))
            assert e2 < 2 * tol_real, f"{what} {key} sum of squares: rel {e2:.3e}"
    return report


# ---------------------------------------------------------------------------
# the same outputs from the numpy oracle and from the CUDA pipeline
# ---------------------------------------------------------------------------
def oracle_outputs(case: dict, scalars: dict) -> dict:
    """the oracle's restatement of what the reference hands its output plugin"""
    from monofonic_gb300 import ic
    from oracle import lpt_oracle as O
    n, L, order = case["ngrid"], case["boxlen"], case.get("lpt_order", 3)
    lat = LAT[case["lattice"]]
    p = O.cosmo_parameters(COSMO["Omega_m"], COSMO["Omega_b"], COSMO["h"], COSMO["sigma_8"], COSMO["n_s"])
    osc = O.scalars_from(p, scalars["Dplus"], scalars["vfac"], scalars["pnorm"])
    f = O.lpt_potentials(ic.white_noise(n, case["seed"]), L, order, osc, convolver=case.get("convolver", "orszag"),
                         fixing=case.get("fixing", False), inversion=case.get("inversion", False))
    out = {}
    fields = case.get("out", "particles") == "field_lagrangian"
    if case.get("baryons"):
        fb = COSMO["Omega_b"] / COSMO["Omega_m"]
        if fields:
            for d, c in enumerate("xyz"):
                out["dm_d" + c] = O.c2r(O.displacement_k(f, L, d, order, unit=L), n)
                out["dm_v" + c] = O.c2r(O.displacement_k(f, L, d, order, unit=L, vel=True, vfac=osc.vfac), n)
            rho_k = f.wn * O.bc_amplitudes(np.sqrt(sum(k * k for k in O.kgrids(n, L))), osc, None, None, False)[0]
            rho_k[0, 0, 0] = 0
            out["dm_mass"] = (1.0 - fb * O.c2r(rho_k, n)) * (COSMO["Omega_m"] - COSMO["Omega_b"])
            kx, ky, kz = O.kgrids(n, L)
            out["dm_density"] = O.c2r(-(kx * kx + ky * ky + kz * kz) * f.phi, n)
            rho, vel = O.eulerian_fields(f, L, order, osc, 1.0 - fb, vunit=L)
            out["baryon_density"] = rho
            for d, c in enumerate("xyz"):
                out["baryon_v" + c] = vel[d]
        else:
            two = O.two_species_particles(f, L, order, osc, COSMO["Omega_m"], COSMO["Omega_b"], lattice=lat,
                                          lunit=L, vunit=L)
            for sp, (pos, vel, ids, mass) in two.items():
                out[sp + "_pos"], out[sp + "_vel"], out[sp + "_ids"], out[sp + "_mass"] = pos, vel, ids, mass
        return out
    if fields:
        for d, c in enumerate("xyz"):
            out["dm_d" + c] = O.c2r(O.displacement_k(f, L, d, order, unit=L), n)
            out["dm_v" + c] = O.c2r(O.displacement_k(f, L, d, order, unit=L, vel=True, vfac=osc.vfac), n)
        kx, ky, kz = O.kgrids(n, L)
        out["dm_density"] = O.c2r(-(kx * kx + ky * ky + kz * kz) * f.phi, n)
        return out
    if case.get("plt"):
        tabs = O.plt_tables(lat, 64)
        ov = 1 << lat
        pos = np.empty((ov * n ** 3, 3))
        vel = np.empty_like(pos)
        for d in range(3):
            fr = O.c2r(O.displacement_k_plt(f, L, d, order, tabs, unit=L), n)
            pos[:, d] = O.lattice_positions_component(fr, d, lat, L, L)
            fv = O.c2r(O.displacement_k_plt(f, L, d, order, tabs, unit=L, vel=True, vfac=osc.vfac), n)
            vel[:, d] = O.lattice_velocities_component(fv, lat, L)
        out["dm_pos"], out["dm_vel"], out["dm_ids"] = pos, vel, O.particle_ids(n, lat)
        return out
    pos, vel, ids = O.particles(f, L, order, osc.vfac, lattice=lat, lunit=L, vunit=L)
    out["dm_pos"], out["dm_vel"], out["dm_ids"] = pos, vel, ids
    return out


def scalars_struct(scalars: dict, zstart: float):
    """the pipeline's cosmology scalars with the reference's D+, vfac, pnorm"""
    from monofonic_gb300 import ic
    sc = ic.cosmology_scalars(ic.Cosmology(**COSMO), zstart)
    sc.Dplus, sc.vfac, sc.pnorm = scalars["Dplus"], scalars["vfac"], scalars["pnorm"]
    return sc


def gpu_outputs(ctx, case: dict, scalars: dict, precision: str = "f64") -> dict:
    """the CUDA pipeline's outputs for `case` through the C ABI, keyed as the
    reference's capture plugin names them"""
    from monofonic_gb300 import ic
    n, L = case["ngrid"], case["boxlen"]
    fields = case.get("out", "particles") == "field_lagrangian"
    cfg = ic.ICConfig(ngrid=n, boxlen=L, zstart=case["zstart"], lpt_order=case.get("lpt_order", 3),
                      lattice=case["lattice"], precision=precision, convolver=case.get("convolver", "orszag"),
                      fixing=case.get("fixing", False), inversion=case.get("inversion", False),
                      plt=case.get("plt", False), lunit=L, vunit=L, out_kind="fields" if fields else "particles",
                      pos64=True, id64=True, baryons=case.get("baryons", False))
    gen = ic.ICGenerator(ctx, cfg, scalars_struct(scalars, case["zstart"]))
    gen.set_noise_seed(case["seed"])
    out = {}
    try:
        if case.get("baryons"):
            res = gen.run_species()
            if fields:
                disp, vel, _, mass = res["dm"]
                for d, c in enumerate("xyz"):
                    out["dm_d" + c], out["dm_v" + c] = disp[d], vel[d]
                out["dm_mass"] = mass
                rho, bvel, _, _ = res["baryon"]
                out["baryon_density"] = rho
                for d, c in enumerate("xyz"):
                    out["baryon_v" + c] = bvel[d]
            else:
                for sp in ("dm", "baryon"):
                    pos, vel, ids, mass = res[sp]
                    out[sp + "_pos"], out[sp + "_vel"], out[sp + "_ids"], out[sp + "_mass"] = pos, vel, ids, mass
        else:
            pos, vel, ids = gen.run()
            if fields:
                for d, c in enumerate("xyz"):
                    out["dm_d" + c], out["dm_v" + c] = pos[d], vel[d]
            else:
                out["dm_pos"], out["dm_vel"], out["dm_ids"] = pos, vel, ids
        if fields:
            out["_phi_k"] = gen.potential(0)
    finally:
        gen.close()
    return out
