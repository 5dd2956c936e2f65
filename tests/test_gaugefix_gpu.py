"""Coulomb gauge fixing and its batched 3D FFT on the GPU, through the C ABI, against numpy's
FFT, the oracle and the reference's own gauge fixer (golden fixture)."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from soerenpragya3dglasma_gb300 import GlasmaError, Lattice, build

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def mild_config(N, seed, eps=0.02, om=0.2):
    """Weak random field in a random gauge, top z-links the identity (as in tests/golden/make_golden.py)."""
    from tests.golden.make_golden import mild_gauge_config

    return mild_gauge_config(N, seed, eps, om)


# power-of-two lengths (radix-2 kernel) and mixed radix (Stockham: radices 4, 2, 3, 5, other primes by
# their direct DFT): the lengths of the batched events' lattices (48, 96, 160, 250), primes 7 and 97,
# and composites with repeated larger primes (49, 121)
@pytest.mark.parametrize("N", [(8, 8, 16), (4, 16, 32), (6, 5, 7), (2, 3, 12), (48, 96, 160), (250, 3, 97),
                               (49, 121, 10), (160, 48, 250)])
def test_fft3d_matches_numpy(N):
    rng = np.random.default_rng(sum(N))
    X = rng.standard_normal((8, N[2], N[1], N[0])) + 1j * rng.standard_normal((8, N[2], N[1], N[0]))
    with Lattice(N) as lat:
        F = lat.fft3d(X)
        B = lat.fft3d(X, inverse=True)
    ref = np.fft.fftn(X, axes=(1, 2, 3))
    refb = np.fft.ifftn(X, axes=(1, 2, 3)) * (N[0] * N[1] * N[2])
    assert np.max(np.abs(F - ref)) / np.max(np.abs(ref)) < 1e-14
    assert np.max(np.abs(B - refb)) / np.max(np.abs(refb)) < 1e-14


@pytest.mark.parametrize("N", [(8, 8, 16), (16, 4, 32), (6, 5, 7), (48, 96, 160), (250, 3, 97)])
def test_fft3d_f32_matches_numpy(N):
    """The FP32 transform (the gauge fixer's GLASMA_GF_FFT_FP32 path): FP32 rounding, ~1e-7 log2(V)."""
    rng = np.random.default_rng(sum(N) + 1)
    X = (rng.standard_normal((8, N[2], N[1], N[0])) + 1j * rng.standard_normal((8, N[2], N[1], N[0]))).astype(np.complex64)
    with Lattice(N) as lat:
        F = lat.fft3d_f32(X)
        B = lat.fft3d_f32(X, inverse=True)
    Xd = X.astype(np.complex128)
    ref = np.fft.fftn(Xd, axes=(1, 2, 3))
    refb = np.fft.ifftn(Xd, axes=(1, 2, 3)) * (N[0] * N[1] * N[2])
    assert np.max(np.abs(F - ref)) / np.max(np.abs(ref)) < 5e-6
    assert np.max(np.abs(B - refb)) / np.max(np.abs(refb)) < 5e-6


def test_fft_fp32_preconditioner_reaches_the_same_gauge():
    """The acceleration step's transforms in FP32 only perturb each step by ~1e-7 of itself: the
    deviation history follows the FP64 run and the gauge-fixed links agree far below the distance
    still left to convergence."""
    N = (8, 8, 16)
    f = mild_config(N, 9)
    out = {}
    for fp32 in (False, True):
        with Lattice(N) as lat:
            lat.upload("U", f["U"])
            log = lat.coulomb_fix(1.0, 100, tol=1e-12, project_zero_mode=True, fft_fp32=fp32)
            out[fp32] = (log, lat.download("UG"))
    l64, l32 = out[False][0], out[True][0]
    assert len(l64) == len(l32) == 100
    assert np.allclose(l32[:, 1:3], l64[:, 1:3], rtol=1e-4, atol=1e-12)
    assert l32[-1, 1] < 1e-2 * l32[0, 1]
    assert np.max(np.abs(out[True][1] - out[False][1])) < 1e-5


def test_coulomb_matches_reference_golden(golden_dir):
    g = dict(np.load(os.path.join(golden_dir, "coulomb_mild.npz")))
    N, a = tuple(g["cfg_N"]), tuple(g["cfg_a"])
    with Lattice(N, a) as lat:
        lat.upload("U", g["U"])
        lat.upload("E", g["E"])
        log = lat.coulomb_fix(float(g["cfg_alpha"]), int(g["cfg_iters"]))
        G, UG, EG = lat.download("G"), lat.download("UG"), lat.download("EG")
    assert len(log) == len(g["log"])
    assert np.allclose(log, g["log"], rtol=2e-5, atol=1e-6)  # the reference logs 6 digits
    assert np.max(np.abs(G - g["G"])) < 1e-12
    assert np.max(np.abs(UG - g["UG"])) < 1e-12
    assert np.max(np.abs(EG - g["EG"])) < 1e-12


# The reference iteration amplifies rounding quickly once its steps grow (the unnormalised p=0 mode):
# the oracle and the compiled reference themselves drift apart to ~1e-5 by iteration 12.  Parity is
# therefore checked over the first iterations, where the steps are still small.
@pytest.mark.parametrize("N,alpha,iters", [((8, 8, 16), 0.5, 4), ((8, 4, 6), 1.0, 3), ((6, 5, 7), 0.5, 3)])
def test_coulomb_matches_oracle(oracle, N, alpha, iters):
    f = mild_config(N, 9)
    G = O.identity_gauge(N)
    st, olog, UG, EG = oracle.coulomb_fix(f, G, N, (1.0, 1.0, 1.0), alpha, iters)
    assert st == 0
    with Lattice(N) as lat:
        lat.upload("U", f["U"])
        lat.upload("E", f["E"])
        log = lat.coulomb_fix(alpha, iters)
        assert np.allclose(log, olog, rtol=1e-10, atol=1e-13)
        assert np.max(np.abs(lat.download("G") - G)) < 1e-11
        assert np.max(np.abs(lat.download("UG") - UG)) < 1e-11
        assert np.max(np.abs(lat.download("EG") - EG)) < 1e-11


def test_coulomb_state_persists_and_resets(oracle):
    """G carries over between calls (the reference's GaugeTransformation::G) until gauge_reset."""
    N = (6, 6, 8)
    f = mild_config(N, 4)
    G = O.identity_gauge(N)
    oracle.coulomb_fix(f, G, N, (1.0, 1.0, 1.0), 0.5, 3)
    st, olog, _, _ = oracle.coulomb_fix(f, G, N, (1.0, 1.0, 1.0), 0.5, 3)
    with Lattice(N) as lat:
        lat.upload("U", f["U"])
        lat.upload("E", f["E"])
        lat.coulomb_fix(0.5, 3)
        log2 = lat.coulomb_fix(0.5, 3)
        assert np.allclose(log2, olog, rtol=1e-10, atol=1e-13)
        lat.gauge_reset()
        assert np.allclose(lat.download("G"), O.identity_gauge(N))


def test_zero_mode_projection_converges():
    """Documented deviation: with the p=0 mode projected out the iteration settles instead of
    drifting (the reference keeps that mode unnormalised)."""
    N = (8, 8, 16)
    f = mild_config(N, 9)
    with Lattice(N) as lat:
        lat.upload("U", f["U"])
        log = lat.coulomb_fix(1.0, 150, tol=1e-12, project_zero_mode=True)
    assert log[-1, 1] < 1e-3 * log[0, 1]


def test_unitarity_guard_returns_status_instead_of_exiting():
    """A corrupted link (NaN) trips the update guard; the call returns GLASMA_ERR_NUMERICAL where
    the reference would exit, and the handle stays usable."""
    N = (6, 6, 8)
    f = O.random_fields(N, 77, link_amp=0.2)
    bad = f["U"].copy()
    bad[3, 2, 1, 0, 0, 0] = np.nan
    with Lattice(N) as lat:
        lat.upload("U", bad)
        with pytest.raises(GlasmaError) as ei:
            lat.coulomb_fix(0.5, 5)
        assert ei.value.status == 5
        lat.upload("U", f["U"])
        lat.gauge_reset()
        assert len(lat.coulomb_fix(0.5, 2)) == 2


def _coulomb_mv(golden_dir):
    g = dict(np.load(os.path.join(golden_dir, "coulomb_mv.npz")))
    return g, tuple(int(v) for v in g["cfg_N"]), tuple(g["cfg_a"]), float(g["cfg_alpha"])


def test_reference_iteration_on_mv_state_exits_like_the_reference(golden_dir):
    """On an evolved MV collision the reference's own iteration leaves SU(3) and exits on its guard
    (golden: the compiled reference run to its stop rule).  The GPU follows its full-precision log
    while the iteration is well conditioned and returns GLASMA_ERR_NUMERICAL where the reference
    calls exit(0); later iterations amplify rounding (tests/test_oracle_golden.py has the control)."""
    g, N, a, alpha = _coulomb_mv(golden_dir)
    with Lattice(N, a) as lat:
        lat.upload("U", g["s_U"])
        lat.upload("E", g["s_E"])
        log = lat.coulomb_fix(alpha, 5)
        ref = g["s_log"][:5]
        assert np.max(np.abs(log[:, 1:] - ref[:, 1:]) / np.abs(ref[:, 1:])) < 1e-10
        lat.gauge_reset()
        with pytest.raises(GlasmaError) as ei:
            lat.coulomb_fix(alpha, 1000)
        assert ei.value.status == 5 and 5 < len(ei.value.log) < 1000


@pytest.mark.parametrize("fft_fp32", [False, True])
def test_open_z_converges_on_reference_state(oracle, golden_dir, fft_fp32):
    """GLASMA_GF_OPEN_Z on the state the reference fails on: converges to the reference's own stop
    rule (max |Delta| <= 1e-15), and the gauge-fixed fields equal the oracle's converged ones."""
    g, N, a, alpha = _coulomb_mv(golden_dir)
    f = {"U": g["s_U"].copy(), "E": g["s_E"].copy()}
    G = O.identity_gauge(N)
    st, olog, UG, EG = oracle.coulomb_fix(f, G, N, a, alpha, 1000, flags=O.GF_OPEN_Z)
    assert st == 0 and olog[-1, 1] <= 1e-15
    with Lattice(N, a) as lat:
        lat.upload("U", f["U"])
        lat.upload("E", f["E"])
        log = lat.coulomb_fix(alpha, 1000, open_z=True, fft_fp32=fft_fp32)
        assert log[-1, 1] <= 1e-15 and len(log) < 1000
        Gg, UGg, EGg = lat.download("G"), lat.download("UG"), lat.download("EG")
    if fft_fp32:
        # the Coulomb gauge is unique up to a global rotation R, and the FP32 rounding of the transforms
        # (of sum_x Delta, in the p = 0 mode) moves the iteration along it: G_gpu(x) = R G_oracle(x) with
        # one R for every site, close to the identity
        Mg, Mo = O.links_as_matrices(Gg)[1:-1], O.links_as_matrices(G)[1:-1]
        R = Mg @ np.swapaxes(Mo.conj(), -1, -2)
        assert np.max(np.abs(R - R[0, 0, 0])) < 1e-10 and np.max(np.abs(R[0, 0, 0] - np.eye(3))) < 1e-5
    else:
        assert np.max(np.abs(UGg - UG)) < 1e-10
        assert np.max(np.abs(EGg - EG)) < 1e-10 * np.max(np.abs(EG))
        assert np.max(np.abs(Gg - G)) < 1e-10
        # theta = <Delta^2> history, while it is above the rounding floor
        th, oth = log[:, 2] ** 2, olog[:, 2] ** 2
        m = min(len(th), len(oth))
        k = oth[:m] > 1e-20
        assert np.allclose(th[:m][k], oth[:m][k], rtol=1e-6)


def test_open_z_converged_fields_match_oracle_16x16x32(oracle, golden_dir):
    """16x16x32 MV collision built and evolved on the GPU (40 steps from the charges of the golden
    16x16x32 case), then Coulomb-fixed with GLASMA_GF_OPEN_Z through theta < 1e-10 to the reference's
    stop rule; the oracle runs the same variant on the downloaded fields.  Converged UG, EG and theta
    agree to 1e-10 (a converged gauge is an attractive fixed point: rounding does not grow)."""
    g, _, a, alpha = _coulomb_mv(golden_dir)
    N = tuple(int(v) for v in g["cfg_N_large"])
    n = 8 * N[0] * N[1]
    zl, zr = g["l_gauss_in"][:n], g["l_gauss_in"][n:]
    dt = float(g["cfg_dt"])
    with Lattice(N, a) as lat:
        lat.mv_init(zl, zr, qs=(float(g["cfg_qs"]),) * 2, centers=(N[2] // 2 - N[2] // 4, N[2] // 2 + N[2] // 4),
                    sigma=float(g["cfg_sigma"]), lam=float(g["cfg_lam"]), meff=float(g["cfg_meff"]), dt=dt)
        lat.step(dt, int(g["cfg_steps_large"]))
        f = lat.download_fields()
        log = lat.coulomb_fix(alpha, 2000, open_z=True)
        UGg, EGg = lat.download("UG"), lat.download("EG")
    G = O.identity_gauge(N)
    st, olog, UG, EG = oracle.coulomb_fix(f, G, N, a, alpha, 2000, flags=O.GF_OPEN_Z)
    assert st == 0 and olog[-1, 1] <= 1e-15 and log[-1, 1] <= 1e-15
    th, oth = log[:, 2] ** 2, olog[:, 2] ** 2
    assert abs(int(np.argmax(th < 1e-10)) - int(np.argmax(oth < 1e-10))) <= 1 and np.argmax(oth < 1e-10) < 300
    m = min(len(th), len(oth))
    k = oth[:m] > 1e-20
    assert np.allclose(th[:m][k], oth[:m][k], rtol=1e-6)
    assert np.max(np.abs(UGg - UG)) < 1e-10
    assert np.max(np.abs(EGg - EG)) < 1e-10 * np.max(np.abs(EG))


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_charge_transformation_matches_oracle(oracle, precision):
    """glasma_transform_charge (PERFORM_COLOR_CHARGE_TRANSFORMATION, S/CALC/GaugeTransformation.cpp:28-31)
    with an uploaded G and with the G a gauge-fixing run leaves, against the oracle; the handle's own
    currents are left as they were."""
    from tests.test_oracle_golden import random_gauge

    N = (8, 6, 10)
    f = O.random_fields(N, 77)
    G = random_gauge(N, 78)
    tol = 1e-14 if precision == "fp64" else 2e-7
    with Lattice(N, precision=precision) as lat:
        lat.upload_fields(f)
        lat.upload("G", G)
        Gd = lat.download("G")
        for k in ("Jp", "Jm", "JpStat", "JmStat"):
            J = lat.download(k)
            got = lat.transform_charge(k)
            want = oracle.transform_charge(Gd, J, N)
            assert np.max(np.abs(got - want)) < tol * max(1.0, np.max(np.abs(want))), k
            assert np.array_equal(lat.download(k), J), k
        with pytest.raises(ValueError):
            lat.transform_charge("E")
        if precision != "fp64":
            return
        # after gauge fixing: the fixer's G
        lat.gauge_reset()
        lat.coulomb_fix(0.5, 5, open_z=True)
        Gd = lat.download("G")
        got = lat.transform_charge("JpStat")
        want = oracle.transform_charge(Gd, lat.download("JpStat"), N)
        assert np.max(np.abs(got - want)) < tol * max(1.0, np.max(np.abs(want)))


def test_mixed_precision_sweeps_reach_the_fp64_gauge(oracle, golden_dir):
    """GLASMA_GF_MIXED with the open-z functional on the reference's MV state: FP32 sweeps until the
    maximum deviation is <= 1e-5 (or stalls), then FP64 sweeps to the reference's stop rule.  It
    converges to the gauge the FP64 iteration reaches (the oracle's converged run), up to one global
    rotation R close to the identity (the FP32 sweeps move the iterate along the gauge's global
    freedom): G_mixed(x) = R G_oracle(x) at every site, and the gauge-fixed fields' gauge-invariant
    content (theta, the functional) matches."""
    g, N, a, alpha = _coulomb_mv(golden_dir)
    f = {"U": g["s_U"].copy(), "E": g["s_E"].copy()}
    G = O.identity_gauge(N)
    st, olog, UG, EG = oracle.coulomb_fix(f, G, N, a, alpha, 1000, flags=O.GF_OPEN_Z)
    assert st == 0
    with Lattice(N, a) as lat:
        lat.upload("U", f["U"])
        lat.upload("E", f["E"])
        log = lat.coulomb_fix(alpha, 1000, open_z=True, mixed=True)
        Gg, UGg = lat.download("G"), lat.download("UG")
    assert log[-1, 1] <= 1e-15 and len(log) < 1000
    n32 = int(np.argmax(log[:, 1] <= 1e-5))  # the FP32 sweeps end at the first row at or below 1e-5
    assert 0 < n32 < len(log) - 1
    Mg, Mo = O.links_as_matrices(Gg)[1:-1], O.links_as_matrices(G)[1:-1]
    R = Mg @ np.swapaxes(Mo.conj(), -1, -2)
    assert np.max(np.abs(R - R[0, 0, 0])) < 1e-9 and np.max(np.abs(R[0, 0, 0] - np.eye(3))) < 1e-3
    # the final functional (sum Re tr UG / V) is invariant under R
    assert abs(log[-1, 6] - olog[-1, 6]) < 1e-12 * abs(olog[-1, 6])
    with Lattice(N, a, precision="fp32") as lat:
        lat.upload("U", f["U"])
        with pytest.raises(GlasmaError):
            lat.coulomb_fix(alpha, 10, open_z=True, mixed=True)
