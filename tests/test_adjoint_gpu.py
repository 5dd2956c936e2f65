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
