"""The plain-method configuration at its full size on the GPU: a 32x32x128 collision of two MV nuclei
(g^2 mu 0.5, m 0.2, centres 40/88, dt 0.125), 200 leapfrog steps, the bulk observables and the
Gauss-law violation every 10 steps (the cadence of S/Simulation.cpp:251-281, made denser).

* sigma_z 5 against the reference's own run (golden `config1_collision.npz`, compiled reference): at
  the asked sigma_z 4 the reference's initial-condition code exits (its eigen-decomposition of the
  ~1e-100 profile slices far from a nucleus fails), which the fixture records;
* sigma_z 4 against the oracle, which evolves the GPU's initial state on the CPU;
* FP32 (reunitarised every 16 steps) against FP64 from the same FP32-rounded start, per observable.
"""
import os

import numpy as np
import pytest

from oracle import oracle as O
from soerenpragya3dglasma_gb300 import Lattice, build

pytestmark = pytest.mark.gpu

BULK_NAMES = ("T00", "TXX", "TYY", "TZZ", "ELECTRIC", "MAGNETIC")  # out[9..14]


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


@pytest.fixture(scope="module")
def golden(golden_dir):
    return dict(np.load(os.path.join(golden_dir, "config1_collision.npz")))


def _setup(g, sigma):
    N = tuple(int(v) for v in g["cfg_N"])
    n = 8 * N[0] * N[1]
    zl, zr = g["gauss_in"][:n], g["gauss_in"][n:2 * n]
    kw = dict(qs=(float(g["cfg_qs"]),) * 2, centers=tuple(int(c) for c in g["cfg_centers"]), sigma=sigma,
              lam=float(g["cfg_lam"]), meff=float(g["cfg_meff"]), dt=float(g["cfg_dt"]))
    return N, zl, zr, kw


def _measure_run(lat, dt, steps, every):
    bulk, gauss, unit = [], [], []
    for k in range(steps // every + 1):
        if k:
            lat.step(dt, every)
        bulk.append(lat.bulk())
        gauss.append(lat.gauss())
        unit.append(lat.unitarity())
    return np.array(bulk), np.array(gauss), np.array(unit)


@pytest.mark.parametrize("method", ["plaquette", "two_pass"])
def test_config1_matches_reference_golden(golden, method):
    g = golden
    N, zl, zr, kw = _setup(g, float(g["cfg_sigma"]))
    with Lattice(N, tuple(g["cfg_a"])) as lat:
        lat.set_step_method(method)
        lat.mv_init(zl, zr, **kw)
        bulk, gauss, unit = _measure_run(lat, kw["dt"], int(g["cfg_steps"]), int(g["cfg_every"]))
    # energy-density sums (T00, pressures, electric and magnetic parts) every 10 steps, relative to the
    # energy (the transverse pressures nearly cancel at t = 0).  The two initial states (the GPU's MV
    # construction and the reference's per-slice eigen-decomposition exponentials) agree to ~1e-13 in
    # the links, but in the dilute regions 3 - ReTr P is ~1e-6, so the magnetic energy of the start
    # already differs by ~1e-9: the bar here is 1e-8 (the evolution itself is held to 1e-10 against the
    # oracle from one shared start below, and to 1e-12 against the reference on its golden steps)
    rb = np.abs(bulk[:, 9:15] - g["bulk"][:, 9:15]) / np.abs(g["bulk"][:, 9:10])
    assert rb.max() < 1e-8, rb.max(axis=0)
    # the Gauss-law violation (it grows from 1e-17 to ~5e-8 over the run at the open z boundaries)
    assert np.allclose(gauss, g["gauss"], rtol=1e-5, atol=1e-14), np.abs(gauss / g["gauss"] - 1).max(axis=0)
    # links stay unitary as closely as the reference keeps them (its own reach 2.7e-12)
    assert np.all(unit[:, 0] < 1e-11) and np.all(g["unitarity"][:, 0] < 1e-11)


def test_config1_asked_width_matches_oracle(oracle, golden):
    """sigma_z 4, where the reference itself exits: the GPU's initial state, evolved by the GPU and by
    the oracle (the reference's update restated; pinned on its golden steps), 200 steps."""
    g = golden
    N, zl, zr, kw = _setup(g, float(g["cfg_sigma_asked"]))
    a = tuple(g["cfg_a"])
    steps, every = int(g["cfg_steps"]), int(g["cfg_every"])
    with Lattice(N, a) as lat:
        lat.mv_init(zl, zr, **kw)
        f = lat.download_fields()
        bulk, gauss, _ = _measure_run(lat, kw["dt"], steps, every)
    ob, og = [], []
    for k in range(steps // every + 1):
        if k:
            oracle.update(f, N, a, kw["dt"], every)
        ob.append(oracle.bulk(f, N, a))
        og.append(oracle.gauss(f, N, a))
    ob, og = np.array(ob), np.array(og)
    rb = np.abs(bulk[:, 9:15] - ob[:, 9:15]) / np.abs(ob[:, 9:10])
    assert rb.max() < 1e-10, rb.max(axis=0)
    # the Gauss violation is itself made of rounding at first (1e-17 at the start, 1e-13 after 10 steps)
    # and grows to ~2e-8 at the open boundaries; two exponentials equal to 1e-16 (the GPU's FP64 power
    # series, the oracle's closed form) move it by ~1e-7 of itself
    assert np.allclose(gauss, og, rtol=1e-6, atol=1e-14), np.abs(gauss / og - 1).max(axis=0)


def test_config1_fp32_error_per_observable(golden):
    """FP32 links, E and currents (reunitarised every 16 steps, FP64 reductions) against FP64 from the
    same FP32-rounded initial state, at sigma_z 4: the error of each observable after 200 steps, beside
    the floor that the FP32 rounding of the start alone sets (FP64 from the FP32-rounded start against
    FP64 from the exact one)."""
    g = golden
    N, zl, zr, kw = _setup(g, float(g["cfg_sigma_asked"]))
    with Lattice(N) as lat:
        lat.mv_init(zl, zr, **kw)
        f0 = lat.download_fields()
    f32 = {k: (v.astype(np.complex64).astype(np.complex128) if np.iscomplexobj(v)
               else v.astype(np.float32).astype(np.float64)) for k, v in f0.items()}
    out = {}
    for tag, prec, start in (("fp64", "fp64", f32), ("fp32", "fp32", f32), ("fp64_exact", "fp64", f0)):
        with Lattice(N, precision=prec, reunitarize_every=16 if prec == "fp32" else 0) as lat:
            lat.upload_fields(start)
            lat.step(kw["dt"], int(g["cfg_steps"]), save_uold=False)
            out[tag] = (lat.bulk(), lat.gauss())
    b64, b32, bex = out["fp64"][0], out["fp32"][0], out["fp64_exact"][0]
    # relative to the energy (the pressures are differences of nearly equal parts)
    err = {n: abs(b32[9 + i] - b64[9 + i]) / abs(b64[9]) for i, n in enumerate(BULK_NAMES)}
    floor = {n: abs(bex[9 + i] - b64[9 + i]) / abs(b64[9]) for i, n in enumerate(BULK_NAMES)}
    print("FP32 vs FP64 after 200 steps (relative to T00):", err, "floor of the FP32-rounded start:", floor,
          "gauss fp32/fp64:", out["fp32"][1], out["fp64"][1])
    # measured on GB300: the energy 1e-5 from FP64, below the 3e-5 that the rounding of the start alone
    # causes; the other sums within 1e-4 of the energy
    assert err["T00"] < max(1e-6, 2 * floor["T00"]), (err, floor)
    assert max(err.values()) < 1e-4, (err, floor)
    assert out["fp32"][1][1] < 1e-5
