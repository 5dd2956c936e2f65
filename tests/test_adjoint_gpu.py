"""Adjoint leapfrog: gradients of a late-time observable with respect to the initial E field and
colour currents, checked against central finite differences (eps = 1e-6, FP64) along random
directions, and across checkpoint spacings (time-reversed integration vs stored states)."""
import numpy as np
import pytest

from oracle import oracle as O
from soerenpragya3dglasma_gb300 import Lattice, build

pytestmark = pytest.mark.gpu

N, A, DT, STEPS = (6, 6, 12), (1.0, 1.0, 1.0), 0.1, 8
Z0, Z1 = 3, 9
GRAD_FIELDS = ("E", "Jp", "Jm", "JpStat", "JmStat")


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def initial():
    f = O.random_fields(N, 555, link_amp=0.25, e_amp=0.3, j_amp=0.1)
    return f


def objective_after(fields, form):
    with Lattice(N, A) as lat:
        lat.upload_fields(fields)
        lat.step(DT, STEPS, save_uold=False)
        return lat.objective(Z0, Z1, form)


def direction(seed, which):
    rng = np.random.default_rng(seed)
    d = {}
    for k in which:
        v = rng.standard_normal(O.new_fields(N)[k].shape)
        O.sync_ghosts(v)
        d[k] = v
    return d


def interior_dot(grads, d):
    return sum(float(np.sum(grads[k][1:-1] * d[k][1:-1])) for k in d)


@pytest.mark.parametrize("form", [Lattice.PL_OVER_PT, Lattice.ENERGY])
@pytest.mark.parametrize("which,seed", [(("E",), 1), (("Jp", "JpStat"), 2), (("Jm", "JmStat"), 3),
                                        (("E", "Jp", "Jm", "JpStat", "JmStat"), 4)])
def test_gradient_matches_central_differences(form, which, seed):
    f0 = initial()
    with Lattice(N, A) as lat:
        lat.upload_fields(f0)
        L0, grads = lat.adjoint(DT, STEPS, Z0, Z1, form, checkpoint_every=3)
        after = lat.download_fields()
    for k in ("U", "E", "Jp", "JpStat"):  # the handle is left in its initial state
        assert np.max(np.abs(after[k] - f0[k])) < 1e-12, k
    assert abs(L0 - objective_after(f0, form)) <= 1e-12 * abs(L0)
    d = direction(seed, which)
    eps = 1e-6
    fp, fm = O.copy_fields(f0), O.copy_fields(f0)
    for k in d:
        fp[k] = f0[k] + eps * d[k]
        fm[k] = f0[k] - eps * d[k]
    fd = (objective_after(fp, form) - objective_after(fm, form)) / (2 * eps)
    ad = interior_dot(grads, d)
    assert abs(fd - ad) <= 1e-5 * max(abs(fd), 1e-3 * abs(L0)), (fd, ad)


def test_checkpoint_spacing_does_not_change_gradient():
    f0 = initial()
    out = []
    for every in (1, 4, 100):
        with Lattice(N, A) as lat:
            lat.upload_fields(f0)
            out.append(lat.adjoint(DT, STEPS, Z0, Z1, Lattice.PL_OVER_PT, checkpoint_every=every)[1])
    for k in GRAD_FIELDS:
        scale = np.max(np.abs(out[0][k]))
        assert np.max(np.abs(out[1][k] - out[0][k])) <= 1e-10 * scale, k
        assert np.max(np.abs(out[2][k] - out[0][k])) <= 1e-9 * scale, k


def _rel_l2(a, b):
    return float(np.linalg.norm(a[1:-1] - b[1:-1]) / np.linalg.norm(b[1:-1]))


def test_fp32_adjoint_follows_the_fp64_adjoint():
    """On an FP32 lattice the adjoint runs in FP32 end to end (forward, time-reversed reconstruction,
    vector-Jacobian products).  Started from the same fields (rounded to FP32 for both), its objective
    and gradients agree with the FP64 adjoint's to FP32 accuracy."""
    f0 = initial()
    f32 = {k: (v.astype(np.complex64).astype(np.complex128) if np.iscomplexobj(v)
               else v.astype(np.float32).astype(np.float64)) for k, v in f0.items()}
    res = {}
    for prec in ("fp64", "fp32"):
        with Lattice(N, A, precision=prec) as lat:
            lat.upload_fields(f32)
            res[prec] = lat.adjoint(DT, STEPS, Z0, Z1, Lattice.PL_OVER_PT, checkpoint_every=3)
    (l64, g64), (l32, g32) = res["fp64"], res["fp32"]
    assert abs(l32 - l64) <= 1e-5 * abs(l64)
    errs = {k: _rel_l2(g32[k], g64[k]) for k in GRAD_FIELDS}
    assert all(e < 2e-4 for e in errs.values()), errs


@pytest.mark.parametrize("link_amp", [0.25, 1e-3])
def test_fp32_objective_matches_fp64_measurement(link_amp):
    """The objective of the same fields on both lattices.  Weak fields (links within 1e-3 of the
    identity, as in the dilute central region of a late collision) are the hard case for FP32: the
    plaquette term is formed without cancellation against 3 (the bulk energy's identity)."""
    f0 = O.random_fields(N, 555, link_amp=link_amp, e_amp=0.3 * link_amp, j_amp=0.1)
    f32 = {k: (v.astype(np.complex64).astype(np.complex128) if np.iscomplexobj(v)
               else v.astype(np.float32).astype(np.float64)) for k, v in f0.items()}
    vals = []
    for prec in ("fp64", "fp32"):
        with Lattice(N, A, precision=prec) as lat:
            lat.upload_fields(f32)
            vals.append(lat.objective(Z0, Z1, Lattice.PL_OVER_PT))
    # weak fields: the plaquette differences A - B (~1e-3) carry FP32 rounding of ~1e-7
    tol = 1e-5 if link_amp > 0.1 else 1e-3
    assert abs(vals[1] - vals[0]) <= tol * abs(vals[0]), vals
