"""The Los Alamos and Jacobi Coulomb gauge fixers on the GPU, through the C ABI
(glasma_coulomb_fix_algorithm), against the reference's own updates (golden fixture) and the
oracle, plus the properties the algorithms guarantee."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from soerenpragya3dglasma_gb300 import GlasmaError, Lattice, build

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def mild_config(N, seed):
    from tests.golden.make_golden import mild_gauge_config

    return mild_gauge_config(N, seed)


def _fix(N, a, f, alg, param, iters, seed=0, tol=1e-15, precision="fp64"):
    with Lattice(N, a, precision=precision) as lat:
        lat.upload("U", f["U"])
        lat.upload("E", f["E"])
        log = lat.coulomb_fix(param, iters, tol=tol, algorithm=alg, seed=seed)
        return log, lat.download("G"), lat.download("UG"), lat.download("EG")


@pytest.mark.parametrize("tag,alg,param", [("la0", "los_alamos", 0.0), ("la5", "los_alamos", 0.5),
                                           ("jac", "jacobi", 0.3)])
def test_local_fixers_match_reference_golden(golden_dir, tag, alg, param):
    g = dict(np.load(os.path.join(golden_dir, "coulomb_local.npz")))
    N, a = tuple(int(v) for v in g["cfg_N"]), tuple(g["cfg_a"])
    log, G, UG, EG = _fix(N, a, {"U": g["U"], "E": g["E"]}, alg, param, int(g["cfg_iters"]),
                          seed=int(g["cfg_draw_seed"]))
    assert len(log) == len(g[tag + "_log"])
    assert np.allclose(log, g[tag + "_log"], rtol=1e-10, atol=1e-13)
    for k, v in (("G", G), ("UG", UG), ("EG", EG)):
        assert np.max(np.abs(v - g[tag + "_" + k])) < 1e-12, k


# odd extents (checkerboard neighbours of equal parity across the periodic x/y seam), the thinnest
# lattice a handle allows, anisotropic spacings
@pytest.mark.parametrize("N,a", [((6, 5, 7), (1.0, 1.0, 1.0)), ((8, 8, 4), (1.0, 0.8, 1.3)),
                                 ((5, 3, 2), (1.0, 1.0, 1.0)), ((7, 7, 9), (0.9, 1.0, 1.1))])
@pytest.mark.parametrize("alg,param,seed", [("los_alamos", 0.0, 0), ("los_alamos", 0.6, 3), ("jacobi", 0.3, 0)])
def test_local_fixers_match_oracle(oracle, N, a, alg, param, seed):
    iters = 5
    f = mild_config(N, 13)
    G = O.identity_gauge(N)
    st, olog, oUG, oEG = oracle.coulomb_fix_local(f, G, N, a, alg, param, iters, seed=seed)
    assert st == 0
    log, dG, dUG, dEG = _fix(N, a, f, alg, param, iters, seed=seed)
    assert np.allclose(log, olog, rtol=1e-10, atol=1e-13)
    assert np.max(np.abs(dG - G)) < 1e-12
    assert np.max(np.abs(dUG - oUG)) < 1e-12
    assert np.max(np.abs(dEG - oEG)) < 1e-12


def test_los_alamos_functional_increases_and_over_relaxation_converges_faster():
    """Each Los Alamos sweep maximises the local gauge functional Re tr w, so without over-relaxation
    the logged functional never decreases; with over-relaxation (probability 0.7) the deviation falls
    faster (two orders of magnitude in 60 iterations on this lattice)."""
    N = (8, 8, 8)
    f = mild_config(N, 9)
    log0 = _fix(N, (1.0, 1.0, 1.0), f, "los_alamos", 0.0, 30)[0]
    assert np.all(np.diff(log0[:, 6]) > -1e-12)
    log7 = _fix(N, (1.0, 1.0, 1.0), f, "los_alamos", 0.7, 60, seed=5)[0]
    assert log7[-1, 1] < 1e-4 * log7[0, 1]
    assert log7[-1, 1] < 0.1 * _fix(N, (1.0, 1.0, 1.0), f, "los_alamos", 0.0, 60)[0][-1, 1]


def test_gauge_carries_over_between_calls(oracle):
    """G persists in the handle (the reference's GaugeTransformation::G); the draws restart with the
    iteration count of each call, in the oracle as on the device."""
    N = (6, 6, 8)
    f = mild_config(N, 4)
    G = O.identity_gauge(N)
    oracle.coulomb_fix_local(f, G, N, (1.0, 1.0, 1.0), "los_alamos", 0.5, 3, seed=9)
    st, olog, _, _ = oracle.coulomb_fix_local(f, G, N, (1.0, 1.0, 1.0), "jacobi", 0.3, 3)
    with Lattice(N) as lat:
        lat.upload("U", f["U"])
        lat.upload("E", f["E"])
        lat.coulomb_fix(0.5, 3, algorithm="los_alamos", seed=9)
        log = lat.coulomb_fix(0.3, 3, algorithm="jacobi")
        assert np.allclose(log, olog, rtol=1e-10, atol=1e-13)
        assert np.max(np.abs(lat.download("G") - G)) < 1e-12


def test_fp32_storage_follows_fp64():
    """An FP32 lattice stores G, UG and EG in FP32 (the arithmetic stays FP64): the first iterations
    follow the FP64 history to FP32 rounding."""
    N = (8, 8, 8)
    f = mild_config(N, 9)
    for alg, param in (("los_alamos", 0.0), ("jacobi", 0.3)):
        l64 = _fix(N, (1.0, 1.0, 1.0), f, alg, param, 6)[0]
        l32 = _fix(N, (1.0, 1.0, 1.0), f, alg, param, 6, precision="fp32")[0]
        assert np.allclose(l32[:, 1:3], l64[:, 1:3], rtol=1e-4, atol=1e-6), alg


def test_invalid_arguments_return_a_status():
    with Lattice((4, 4, 4)) as lat:
        assert lat.lib.glasma_coulomb_fix_algorithm(lat.h, 7, 0.5, 0, 3, 1e-15, 0, None, None) == 1
        with pytest.raises(GlasmaError, match="Fourier update only"):
            lat.coulomb_fix(0.0, 3, algorithm="los_alamos", fft_fp32=True)
        # identity links are already in Coulomb gauge: a negative tolerance forces both iterations
        assert len(lat.coulomb_fix(0.0, 2, tol=-1.0, algorithm="los_alamos")) == 2
