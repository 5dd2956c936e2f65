"""The plaquette method in one launch per step (GLASMA_STEP_MARCH: blocks own (x, y) tiles and march
along z, the rotated force terms handed over in shared memory and registers): every field, ghost slices
and UOld included, bit-identical to the two-kernel plaquette method, for any chunk of slices per block,
tiles that do not divide the lattice, and 12-real links; and against the oracle."""
import numpy as np
import pytest

from oracle import oracle as O
from soerenpragya3dglasma_gb300 import Lattice, build

pytestmark = pytest.mark.gpu

FIELDS = O.FIELD_NAMES


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


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
def test_march_equals_plaquette_method_bit_for_bit(precision, reals, N):
    f = O.random_fields(N, 31)
    a = (1.0, 1.1, 0.9)
    ref = _run(f, N, a, precision, reals, "plaquette", 5)
    got = _run(f, N, a, precision, reals, "march", 5)
    for k in FIELDS:
        assert np.array_equal(got[k], ref[k]), (k, np.max(np.abs(got[k] - ref[k])))


@pytest.mark.parametrize("chunk", [1, 3, 100])
def test_march_chunk_does_not_change_the_fields(chunk):
    N = (12, 10, 9)
    f = O.random_fields(N, 32)
    ref = _run(f, N, (1.0, 1.0, 1.0), "fp32", 18, "plaquette", 4)
    got = _run(f, N, (1.0, 1.0, 1.0), "fp32", 18, "march", 4, chunk=chunk)
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
        assert np.array_equal(got[k], ref[k]), k


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
