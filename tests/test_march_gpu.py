"""The plaquette method in one launch per step (GLASMA_STEP_MARCH: blocks own (x, y) tiles and march
along z, the rotated force terms handed over in shared memory and registers): every field, ghost slices
and UOld included, equal to the two-kernel plaquette method up to rounding (the same terms summed in the
same order; the compiler contracts a few products into fused multiply-adds differently in the two
kernels: FP64 1e-13, FP32 2e-5 after 5 steps of hot random links, as between the other methods), for
any chunk of slices per block, tiles that do not divide the lattice, and 12-real links; and against
the oracle."""
import numpy as np
import pytest

from oracle import oracle as O
from soerenpragya3dglasma_gb300 import Lattice, build

pytestmark = pytest.mark.gpu

FIELDS = O.FIELD_NAMES


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def _rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def _run(f, N, a, precision, reals, method, steps, chunk=0, save_uold=True):
    kw = dict(reunitarize_every=3) if precision == "fp32" else {}
    with Lattice(N, a, precision=precision, **kw) as lat:
        lat.link_reals = reals
        lat.set_step_method(method)
        if chunk:
            lat.set_march_chunk(chunk)
        lat.upload_fields(f)
        lat.step(0.1, steps, save_uold=save_uold)
        assert lat.last_step_method == method
        return lat.download_fields()


@pytest.mark.parametrize("precision,reals", [("fp64", 18), ("fp32", 18), ("fp32", 12)])
@pytest.mark.parametrize("N", [(6, 5, 8), (3, 7, 2), (16, 8, 4), (40, 9, 12), (32, 4, 5)])
def test_march_equals_plaquette_method(precision, reals, N):
    f = O.random_fields(N, 31)
    a = (1.0, 1.1, 0.9)
    ref = _run(f, N, a, precision, reals, "plaquette", 5)
    got = _run(f, N, a, precision, reals, "march", 5)
    tol = 1e-13 if precision == "fp64" else 2e-5
    for k in FIELDS:
        assert _rel(got[k], ref[k]) < tol, (k, _rel(got[k], ref[k]))


@pytest.mark.parametrize("chunk", [1, 3, 100])
def test_march_chunk_does_not_change_the_fields(chunk):
    """The slices per block only move the warm-up slices: the fields are bit-identical."""
    N = (12, 10, 9)
    f = O.random_fields(N, 32)
    ref = _run(f, N, (1.0, 1.0, 1.0), "fp64", 18, "march", 4)
    got = _run(f, N, (1.0, 1.0, 1.0), "fp64", 18, "march", 4, chunk=chunk)
    for k in FIELDS:
        assert np.array_equal(got[k], ref[k]), k


def test_march_without_uold_and_across_calls():
    """Without SaveOldLink the x and y links take one exponential at twice the angle, as in the other
    kernels; odd step counts across calls swap the buffer sets correctly."""
    N = (8, 12, 6)
    f = O.random_fields(N, 33)
    with Lattice(N, precision="fp32") as lat:
        lat.set_step_method("plaquette")
        lat.upload_fields(f)
        lat.step(0.1, 3, save_uold=False)
        lat.step(0.1, 2, save_uold=False)
        ref = lat.download_fields()
    with Lattice(N, precision="fp32") as lat:
        lat.set_step_method("march")
        lat.upload_fields(f)
        lat.step(0.1, 3, save_uold=False)
        lat.step(0.1, 2, save_uold=False)
        got = lat.download_fields()
    for k in FIELDS:
        if k == "UOld":
            continue
        assert _rel(got[k], ref[k]) < 2e-5, k


def test_march_matches_oracle(oracle):
    N, a, dt = (10, 6, 12), (1.0, 0.9, 1.1), 0.1
    f = O.random_fields(N, 34)
    ref = O.copy_fields(f)
    oracle.update(ref, N, a, dt, 4)
    with Lattice(N, a) as lat:
        lat.set_step_method("march")
        lat.upload_fields(f)
        lat.step(dt, 4)
        out = lat.download_fields()
    for k in FIELDS:
        assert np.max(np.abs(out[k] - ref[k])) <= 1e-12 * np.max(np.abs(ref[k])), k
