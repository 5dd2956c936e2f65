"""Parity of the CUDA leapfrog and observables (through the C ABI) with the oracle and with
golden vectors from the reference's own code.  Bar: FP64 relative 1e-10 or better on fields and
observables; FP32 compared against FP64 with the tolerances stated per test."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from soerenpragya3dglasma_gb300 import Lattice, build

pytestmark = pytest.mark.gpu

FIELDS = O.FIELD_NAMES


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def _load(golden_dir, name):
    return dict(np.load(os.path.join(golden_dir, name)))


def _rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def _gpu(fields, N, a, precision="fp64", **kw):
    lat = Lattice(N, a, precision=precision, **kw)
    lat.upload_fields(fields)
    return lat


def test_upload_download_roundtrip_is_bit_exact():
    N = (5, 3, 4)
    f = O.random_fields(N, 3, sync=False)
    f["G"] = O.identity_gauge(N) * (1 + 0.5j)
    with Lattice(N) as lat:
        for k, v in f.items():
            lat.upload(k, v)
        for k, v in f.items():
            assert np.array_equal(lat.download(k), v), k


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_pinned_host_buffers_give_the_same_bytes(precision):
    """Page-locked host buffers are read/written in place by the layout kernels; pageable ones are
    staged.  Both routes must move exactly the same values."""
    torch = pytest.importorskip("torch")
    N = (6, 5, 7)
    f = O.random_fields(N, 4)
    with Lattice(N, precision=precision) as a, Lattice(N, precision=precision) as b:
        for k in ("U", "E", "Jp"):
            pinned = torch.from_numpy(f[k].view(np.float64).copy()).pin_memory()
            a.upload(k, pinned)
            b.upload(k, f[k])
            out_pinned = torch.empty_like(pinned).pin_memory()
            a.download(k, out_pinned)
            out_pageable = b.download(k)
            assert np.array_equal(out_pinned.numpy(), out_pageable.view(np.float64).reshape(out_pinned.shape)), k


@pytest.mark.parametrize("method", ["two_pass", "plaquette"])
@pytest.mark.parametrize("tag,nsteps", [("s1", 1), ("s10", 10)])
def test_leapfrog_matches_reference_golden(golden_dir, tag, nsteps, method):
    g = _load(golden_dir, "leapfrog_random.npz")
    N, a, dt = tuple(g["cfg_N"]), tuple(g["cfg_a"]), float(g["cfg_dt"])
    init = {k: g["init_" + k] for k in FIELDS}
    with _gpu(init, N, a) as lat:
        lat.set_step_method(method)
        lat.step(dt, nsteps)
        assert lat.last_step_method == method
        out = lat.download_fields()
        for k in FIELDS:
            assert _rel(out[k], g[tag + "_" + k]) < 1e-12, k
        assert np.allclose(lat.bulk(), g[tag + "_bulk"], rtol=1e-12, atol=1e-12)
        assert np.allclose(lat.gauss(), g[tag + "_gauss"], rtol=1e-12)
        mx, avg, prof = lat.gauss(sync_first=True, profile=True)
        assert np.allclose(prof, g[tag + "_gauss_profile"], rtol=1e-13, atol=1e-14)
        assert np.allclose(lat.emt_map(), g[tag + "_emt"], rtol=1e-12, atol=1e-13)
        assert lat.unitarity()[0] < 1e-12


@pytest.mark.parametrize("N,a,dt,seed", [((6, 5, 8), (1.0, 1.0, 1.0), 0.125, 11),
                                         ((8, 8, 16), (1.0, 1.1, 0.5), 0.05, 12),
                                         ((3, 7, 2), (1.0, 1.0, 1.0), 0.1, 13)])
@pytest.mark.parametrize("method", ["two_pass", "plaquette"])
def test_leapfrog_matches_oracle(oracle, N, a, dt, seed, method):
    f = O.random_fields(N, seed)
    ref = O.copy_fields(f)
    oracle.update(ref, N, a, dt, 5)
    with _gpu(f, N, a) as lat:
        lat.set_step_method(method)
        lat.step(dt, 5)
        out = lat.download_fields()
    for k in FIELDS:
        assert _rel(out[k], ref[k]) < 1e-12, k


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("N", [(6, 5, 8), (3, 7, 2), (16, 8, 4)])
def test_one_pass_equals_two_pass_bit_exact(precision, N):
    """The one-pass step (second buffer set, static currents one slice up recomputed per site) and
    the two in-place kernels round identically: every field, ghost slices included."""
    f = O.random_fields(N, 21)
    kw = dict(reunitarize_every=3) if precision == "fp32" else {}
    outs = []
    for method in ("one_pass", "two_pass"):
        with _gpu(f, N, (1.0, 1.1, 0.9), precision=precision, **kw) as lat:
            lat.set_step_method(method)
            lat.step(0.1, 7, save_uold=True)
            assert lat.last_step_method == method
            outs.append(lat.download_fields())
    for k in FIELDS:
        assert np.array_equal(outs[0][k], outs[1][k]), k


@pytest.mark.parametrize("tag,nsteps", [("s1", 1), ("s10", 10)])
def test_double_float_force_matches_reference_golden(golden_dir, tag, nsteps):
    """The FP64 plaquette force computed in double-float arithmetic (pairs of floats, ~48-bit
    significand; FP64 fields converted by bits on load and store): the reference's golden fields at
    the FP64 bar, and the native FP64 step to 1e-13."""
    g = _load(golden_dir, "leapfrog_random.npz")
    N, a, dt = tuple(g["cfg_N"]), tuple(g["cfg_a"]), float(g["cfg_dt"])
    init = {k: g["init_" + k] for k in FIELDS}
    outs = {}
    for mode in ("double_float", "native"):
        with _gpu(init, N, a) as lat:
            lat.set_step_method("plaquette")
            lat.fp64_arithmetic = mode
            assert lat.fp64_arithmetic == mode
            lat.step(dt, nsteps)
            outs[mode] = lat.download_fields()
    for k in FIELDS:
        assert _rel(outs["double_float"][k], g[tag + "_" + k]) < 1e-12, k
        assert _rel(outs["double_float"][k], outs["native"][k]) < 1e-13, k


@pytest.mark.parametrize("precision,reals", [("fp64", 18), ("fp32", 18), ("fp32", 12)])
@pytest.mark.parametrize("N", [(6, 5, 8), (3, 7, 2), (16, 8, 4)])
def test_plaquette_method_equals_two_pass(precision, reals, N):
    """The plaquette method sums the same force terms in another order: every field, ghost slices
    included, equal to the two-pass step up to rounding (FP64 1e-13; FP32 2e-5 after 7 steps of hot
    random links)."""
    f = O.random_fields(N, 23)
    kw = dict(reunitarize_every=3) if precision == "fp32" else {}
    outs = []
    for method in ("plaquette", "two_pass"):
        with _gpu(f, N, (1.0, 1.1, 0.9), precision=precision, **kw) as lat:
            lat.link_reals = reals
            lat.set_step_method(method)
            lat.step(0.1, 7, save_uold=True)
            assert lat.last_step_method == method
            outs.append(lat.download_fields())
    tol = 1e-13 if precision == "fp64" else 2e-5
    for k in FIELDS:
        assert _rel(outs[0][k], outs[1][k]) < tol, k


def test_step_method_switch_mid_run(oracle):
    """Odd and even step counts with each method, switching between calls, still follow the oracle."""
    N, dt = (6, 6, 10), 0.1
    f = O.random_fields(N, 22)
    ref = O.copy_fields(f)
    oracle.update(ref, N, (1.0, 1.0, 1.0), dt, 3, save_uold=False)
    oracle.update(ref, N, (1.0, 1.0, 1.0), dt, 2, save_uold=False)
    oracle.update(ref, N, (1.0, 1.0, 1.0), dt, 1, save_uold=False)
    oracle.update(ref, N, (1.0, 1.0, 1.0), dt, 1, save_uold=True)
    with _gpu(f, N, (1.0, 1.0, 1.0)) as lat:
        lat.step(dt, 3, save_uold=False)
        lat.set_step_method("two_pass")
        lat.step(dt, 2, save_uold=False)
        lat.set_step_method("plaquette")
        lat.step(dt, 1, save_uold=False)
        lat.set_step_method("one_pass")
        lat.step(dt, 1, save_uold=True)
        out = lat.download_fields()
    for k in FIELDS:
        assert _rel(out[k], ref[k]) < 1e-12, k


def test_unsynced_ghosts_are_read_as_the_reference_reads_them(oracle):
    """Uploaded ghost slices that are out of date: the reference syncs U at the start of the
    electric update but reads the current ghosts of Jp/Jm as they stand."""
    N, a, dt = (4, 4, 6), (1.0, 1.0, 1.0), 0.1
    f = O.random_fields(N, 21, sync=False)
    ref = O.copy_fields(f)
    oracle.update(ref, N, a, dt, 2)
    with _gpu(f, N, a) as lat:
        lat.step(dt, 2)
        out = lat.download_fields()
    for k in FIELDS:
        assert _rel(out[k], ref[k]) < 1e-12, k


def test_substeps_match_oracle(oracle):
    N, a, dt = (6, 4, 8), (1.0, 0.8, 1.2), 0.1
    f = O.random_fields(N, 31)
    ref = O.copy_fields(f)
    lib = oracle.lib
    with _gpu(f, N, a) as lat:
        # Dynamics::SUNc::Update spelled out sub-step by sub-step
        lat.update_efield(dt)
        lat.update_jstat(dt)
        lat.update_links(0.5 * dt)
        lat.save_old_link()
        lat.update_j(dt)
        lat.update_links(0.5 * dt)
        out = lat.download_fields()
    oracle.update(ref, N, a, dt, 1)
    for k in FIELDS:
        assert _rel(out[k], ref[k]) < 1e-12, k


def test_mv_collision_matches_reference_golden(golden_dir):
    g = _load(golden_dir, "mv_collision.npz")
    N, a, dt = tuple(g["cfg_N"]), tuple(g["cfg_a"]), float(g["cfg_dt"])
    init = {k: g["init_" + k] for k in FIELDS}
    with _gpu(init, N, a) as lat:
        # B^2 sums 4*(3 - ReTr P) with P ~ 1: absolute rounding ~ V * 12 * eps
        assert np.allclose(lat.bulk(), g["t0_bulk"], rtol=1e-12, atol=1e-11)
        assert np.allclose(lat.gauss(), g["t0_gauss"], rtol=1e-10, atol=1e-16)
        lat.step(dt, int(g["cfg_steps"]))
        assert np.allclose(lat.bulk(), g["t8_bulk"], rtol=1e-11, atol=1e-11)
        assert np.allclose(lat.gauss(), g["t8_gauss"], rtol=1e-10, atol=1e-15)
        # the map's entries (~1e-6 here) are slice averages of 3 - ReTr P with P ~ 1: FP64 rounding of
        # the O(1) plaquettes leaves ~1e-14 absolute, whatever the operation order (the link update
        # forms exp(2iQ) once where the reference applies exp(iQ) twice)
        assert np.allclose(lat.emt_map(), g["t8_emt"], rtol=1e-10, atol=1e-13)


def test_observables_match_oracle_on_larger_lattice(oracle):
    N, a = (16, 12, 20), (1.0, 1.0, 0.8)
    f = O.random_fields(N, 41, link_amp=0.2)
    with _gpu(f, N, a) as lat:
        assert np.allclose(lat.bulk(), oracle.bulk(f, N, a), rtol=1e-12, atol=1e-10)
        gm = lat.gauss(profile=True)
        om = oracle.gauss(f, N, a, profile=True)
        assert np.allclose(gm[:2], om[:2], rtol=1e-12)
        assert np.allclose(gm[2], om[2], rtol=1e-12)
        assert np.allclose(lat.emt_map(), oracle.emt_map(f, N, a), rtol=1e-11, atol=1e-13)
        assert np.allclose(lat.unitarity(), oracle.unitarity(f, N), rtol=1e-3, atol=1e-15)


def test_fp32_tracks_fp64(oracle):
    """FP32 storage and arithmetic, FP64 reductions: energy within 1e-6 relative after 20 steps of
    a smooth random field, fields within FP32 rounding growth."""
    N, a, dt = (12, 12, 16), (1.0, 1.0, 1.0), 0.1
    f = O.random_fields(N, 51, link_amp=0.15, e_amp=0.1, j_amp=0.02)
    ref = O.copy_fields(f)
    oracle.update(ref, N, a, dt, 20)
    with _gpu(f, N, a, precision="fp32", reunitarize_every=16) as lat:
        lat.step(dt, 20)
        e32 = lat.bulk()
        out = lat.download_fields()
        umax, _ = lat.unitarity()
    e64 = oracle.bulk(ref, N, a)
    assert abs(e32[9] - e64[9]) / abs(e64[9]) < 1e-6
    assert _rel(out["U"], ref["U"]) < 1e-5
    assert _rel(out["E"], ref["E"]) < 1e-4
    assert umax < 1e-5


@pytest.mark.parametrize("link_amp", [0.02, 0.3])
def test_fp32_bulk_matches_fp64_measurement_of_same_fields(oracle, link_amp):
    """The FP32 energy kernel (plaquette halves in FP32, trace and sums in FP64) against the oracle
    measuring the very same FP32 fields in FP64: per-plane magnetic sums within 1e-6 relative,
    electric sums within 1e-12, also for weak fields where 3 - ReTr(P) is small."""
    N, a = (12, 10, 14), (1.0, 1.0, 1.0)
    f = O.random_fields(N, 53, link_amp=link_amp, e_amp=0.1, j_amp=0.02)
    with _gpu(f, N, a, precision="fp32") as lat:
        got = lat.bulk()
        stored = lat.download_fields()
    want = oracle.bulk(stored, N, a)
    # out[0..2] ESqr, [3..5] BSqr, [6..8] EDotJ, [9..15] T00, TXX, TYY, TZZ, ELECTRIC, MAGNETIC, SOURCE
    for k in (3, 4, 5, 14):  # magnetic sums
        assert abs(got[k] - want[k]) <= 1e-6 * abs(want[k]), k
    for k in (0, 1, 2, 6, 7, 8, 13, 15):  # electric and source sums: FP64 arithmetic on the same floats
        assert abs(got[k] - want[k]) <= 1e-12 * abs(want[k]) + 1e-14, k
    assert abs(got[9] - want[9]) <= 1e-6 * abs(want[9])


def test_fp32_reunitarize_restores_unitarity():
    N = (4, 4, 4)
    f = O.random_fields(N, 61)
    f["U"] = f["U"] * (1 + 1e-3)
    with _gpu(f, N, (1.0, 1.0, 1.0), precision="fp32") as lat:
        assert lat.unitarity()[0] > 1e-3
        lat.reunitarize()
        assert lat.unitarity()[0] < 1e-6


def test_pressure_anisotropy_from_emt_map(oracle):
    N, a = (8, 8, 24), (1.0, 1.0, 1.0)
    f = O.random_fields(N, 91, link_amp=0.25)
    emt = oracle.emt_map(f, N, a)
    z0, z1 = 8, 16
    pl = emt[z0:z1, 3].mean()
    pt = 0.5 * (emt[z0:z1, 1] + emt[z0:z1, 2]).mean()
    with _gpu(f, N, a) as lat:
        r, gl, gt = lat.pressure_anisotropy(z0, z1)
    assert np.allclose([gl, gt, r], [pl, pt, pl / pt], rtol=1e-11)


def test_mv_init_matches_reference_golden(golden_dir):
    """MV collision initial state built on the GPU from the same injected charge fluctuations the
    reference's SetWilsonLines/SingleSheet consumed (golden fixture from the compiled reference)."""
    g = _load(golden_dir, "mv_collision.npz")
    N, a, dt = tuple(g["cfg_N"]), tuple(g["cfg_a"]), float(g["cfg_dt"])
    n = 8 * N[0] * N[1]
    zl, zr = g["gauss_in"][:n], g["gauss_in"][n:2 * n]
    with Lattice(N, a) as lat:
        lat.mv_init(zl, zr, qs=(float(g["cfg_qs"]),) * 2, centers=(int(g["center_left"]), int(g["center_right"])),
                    sigma=float(g["cfg_sigma"]), lam=float(g["cfg_lam"]), meff=float(g["cfg_meff"]), dt=dt)
        out = lat.download_fields()
        for k in FIELDS:
            ref = g["init_" + k]
            assert np.max(np.abs(out[k] - ref)) <= 1e-11 * max(np.max(np.abs(ref)), 1e-3), k
        assert np.allclose(lat.bulk(), g["t0_bulk"], rtol=1e-10, atol=1e-11)


@pytest.mark.parametrize("method", ["two_pass", "plaquette"])
def test_fp32_tracks_fp64_on_a_weak_field_collision(method):
    """An MV collision has dilute regions where the links sit within ~1e-5 of the identity: there FP32
    rounding of the link exponential, of the link stores and of the reunitarisation used to bias the
    state (energy 0.5 % off after a few hundred steps).  From the same FP32-rounded start, FP32 with
    reunitarisation every 16 steps now follows FP64 to the level the initial rounding itself sets."""
    N, dt, steps = (32, 32, 128), 0.125, 200
    rng = np.random.default_rng(2718)
    zl, zr = rng.standard_normal(8 * N[0] * N[1]), rng.standard_normal(8 * N[0] * N[1])
    with Lattice(N) as lat:
        lat.mv_init(zl, zr, qs=(0.5, 0.5), centers=(52, 76), sigma=3.0, lam=1.65, meff=0.2, dt=dt)
        f0 = lat.download_fields()
    f32 = {k: (v.astype(np.complex64).astype(np.complex128) if np.iscomplexobj(v)
               else v.astype(np.float32).astype(np.float64)) for k, v in f0.items()}
    out = {}
    for prec in ("fp64", "fp32"):
        with Lattice(N, precision=prec, reunitarize_every=16 if prec == "fp32" else 0) as lat:
            lat.set_step_method(method)
            lat.upload_fields(f32)
            lat.step(dt, steps, save_uold=False)
            out[prec] = (lat.bulk()[9], lat.unitarity()[0])
    assert abs(out["fp32"][0] - out["fp64"][0]) <= 3e-4 * abs(out["fp64"][0]), out
    assert out["fp32"][1] < 1e-5, out


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_upload_begin_finish(precision):
    """glasma_upload_begin / _finish give the same fields as glasma_upload; kernels enqueued before
    finish see the old fields; a loop that sends the next step's inputs while the current step runs
    ends where the plain loop ends."""
    N, dt = (8, 6, 10), 0.1
    fa = O.random_fields(N, 31)
    fb = O.random_fields(N, 32)
    names = ("U", "E", "Jp", "Jm", "JpStat", "JmStat")
    with Lattice(N, precision=precision) as a, Lattice(N, precision=precision) as b:
        a.upload_fields(fa)
        for k in names:
            b.upload_begin(k, fb[k])
        # nothing converted yet: the handle still holds its creation state
        assert np.allclose(b.download("E"), 0.0)
        b.upload_finish()
        a.upload_fields(fb)
        for k in names:
            assert np.array_equal(a.download(k), b.download(k)), k
    seq, pipe = {}, {}
    with Lattice(N, precision=precision) as a:
        for f in (fa, fb, fa):
            a.upload_fields(f)
            a.step(dt, 1, save_uold=False)
            seq.setdefault("bulk", []).append(a.bulk()[9])
    with Lattice(N, precision=precision) as b:
        plan = [fa, fb, fa]
        for k in names:
            b.upload_begin(k, plan[0][k])
        b.upload_finish()
        for i in range(3):
            if i + 1 < 3:
                for k in names:
                    b.upload_begin(k, plan[i + 1][k])
            b.step(dt, 1, save_uold=False)
            pipe.setdefault("bulk", []).append(b.bulk()[9])
            b.upload_finish()
    assert seq["bulk"] == pipe["bulk"]


@pytest.mark.parametrize("scale", [1e-4, 0.01, 0.05, 0.1, 0.2, 0.4, 1.5, 6.0])
def test_link_exponential_across_its_tiers(oracle, scale):
    """UpdateGaugeLinks alone with E scaled so that the FP64 exponential runs each of its forms (the
    Taylor polynomial for tiny arguments, the 7-, 8-, 11- and 17-term Cayley-Hamilton series below
    c1 = 0.5, the closed form above; scale 0.01 gives c1 in 1e-6..1e-5, 0.1 in 7e-5..9e-4, 0.2 in
    3e-4..4e-3): links against the oracle's exponential at 1e-14."""
    N, a, dt = (6, 4, 8), (1.0, 1.0, 1.0), 1.0
    f = O.random_fields(N, 41)
    f["E"] = f["E"] * scale
    ref = O.copy_fields(f)
    oracle.lib.oracle_update_links(O._ivec(N), O._dvec(a), dt, O._ptr(ref["U"]), O._ptr(ref["E"]))
    with _gpu(f, N, a) as lat:
        lat.update_links(dt)
        U = lat.download("U")
    sl = slice(1, -1)  # interior slices (the sub-step leaves ghost syncs to the caller)
    assert np.max(np.abs(U[sl] - ref["U"][sl])) < 1e-14 * max(1.0, scale)
