"""12-real link storage of the FP32 leapfrog: the step kernels read and write rows 0 and 1 of each
link and form row 2 as conj(row0 x row1).  Bars: the same FP32-vs-FP64 tolerances as full FP32 links;
bit-identical fields from the one-pass and two-pass methods; full SU(3) links between calls."""
import numpy as np
import pytest

from oracle import oracle as O
from soerenpragya3dglasma_gb300 import Lattice, build
from soerenpragya3dglasma_gb300._lib import GlasmaError

pytestmark = pytest.mark.gpu

FIELDS = O.FIELD_NAMES


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def _rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def _fp32(fields, N, a=(1.0, 1.0, 1.0), reals=12, **kw):
    lat = Lattice(N, a, precision="fp32", **kw)
    lat.link_reals = reals
    lat.upload_fields(fields)
    return lat


def _matrices(U):
    """Host links (..., mu, j, i) -> matrices (..., mu, i, j)."""
    return np.swapaxes(U, -1, -2)


def test_link_storage_setting():
    with Lattice((4, 4, 4), precision="fp32") as lat:
        assert lat.link_reals == 18
        lat.link_reals = 12
        assert lat.link_reals == 12
        with pytest.raises(GlasmaError):
            lat.link_reals = 13
        assert lat.link_reals == 12
        lat.link_reals = 18
        assert lat.link_reals == 18
    with Lattice((4, 4, 4), precision="fp64") as lat:
        with pytest.raises(GlasmaError):
            lat.link_reals = 12
        assert lat.link_reals == 18


def test_links12_tracks_fp64(oracle):
    """As full FP32 links: energy within 1e-6 of FP64 after 20 steps of a smooth random field, fields
    within FP32 rounding growth, and within that growth of the 18-real FP32 run."""
    N, a, dt = (12, 12, 16), (1.0, 1.0, 1.0), 0.1
    f = O.random_fields(N, 51, link_amp=0.15, e_amp=0.1, j_amp=0.02)
    ref = O.copy_fields(f)
    oracle.update(ref, N, a, dt, 20)
    e64 = oracle.bulk(ref, N, a)
    out = {}
    for reals in (12, 18):
        with _fp32(f, N, a, reals=reals, reunitarize_every=16) as lat:
            lat.step(dt, 20)
            out[reals] = (lat.bulk(), lat.download_fields(), lat.unitarity()[0])
    e32, f32, umax = out[12]
    assert abs(e32[9] - e64[9]) / abs(e64[9]) < 1e-6
    assert _rel(f32["U"], ref["U"]) < 1e-5
    assert _rel(f32["E"], ref["E"]) < 1e-4
    assert umax < 1e-5
    assert _rel(f32["U"], out[18][1]["U"]) < 1e-5
    assert _rel(f32["E"], out[18][1]["E"]) < 1e-4


@pytest.mark.parametrize("N", [(8, 6, 10), (16, 4, 5)])
def test_links12_one_pass_equals_two_pass_bit_exact(N):
    """Every load forms row 2 with the same expression, so the two step methods round identically
    with 12-real links too: every field, ghost slices included."""
    f = O.random_fields(N, 21)
    outs = []
    for method in ("one_pass", "two_pass"):
        with _fp32(f, N, (1.0, 1.1, 0.9), reunitarize_every=3) as lat:
            lat.set_step_method(method)
            lat.step(0.1, 7, save_uold=True)
            assert lat.last_step_method == method
            outs.append(lat.download_fields())
    for k in FIELDS:
        assert np.array_equal(outs[0][k], outs[1][k]), k


def test_links12_leaves_full_links_between_calls():
    """After a step call every link's row 2 is conj(row0 x row1) of the stored rows (FP32 rounding of
    the products), ghost slices included, and the links are unitary to FP32 precision; UOld, written
    from the full product, is unitary too."""
    N = (8, 8, 6)
    f = O.random_fields(N, 33)
    with _fp32(f, N, reunitarize_every=0) as lat:
        lat.step(0.1, 5, save_uold=True)
        out = lat.download_fields()
        umax = lat.unitarity()[0]
    M = _matrices(out["U"])
    want = np.conj(np.cross(M[..., 0, :], M[..., 1, :]))
    assert np.max(np.abs(M[..., 2, :] - want)) < 1e-6
    assert umax < 1e-5
    W = _matrices(out["UOld"])
    eye = np.eye(3)
    assert np.max(np.abs(W @ np.conj(np.swapaxes(W, -1, -2)) - eye)) < 1e-5


def test_links12_reunitarisation_acts_on_the_stored_rows():
    """Links scaled off SU(3) by 1e-3: the step's reunitarisation projects the two stored rows back,
    and the completed links are unitary to FP32 precision."""
    N = (4, 4, 6)
    f = O.random_fields(N, 61)
    f["U"] = f["U"] * (1 + 1e-3)
    with _fp32(f, N, reunitarize_every=1) as lat:
        assert lat.unitarity()[0] > 1e-3
        lat.step(0.05, 1, save_uold=False)
        assert lat.unitarity()[0] < 1e-5


def test_links12_tracks_fp64_on_a_weak_field_collision():
    """The weak-field MV collision of the full-link FP32 regression test, with 12-real links: from the
    same FP32-rounded start, energy within the same 3e-4 of FP64 after 200 steps."""
    N, dt, steps = (32, 32, 128), 0.125, 200
    rng = np.random.default_rng(2718)
    zl, zr = rng.standard_normal(8 * N[0] * N[1]), rng.standard_normal(8 * N[0] * N[1])
    with Lattice(N) as lat:
        lat.mv_init(zl, zr, qs=(0.5, 0.5), centers=(52, 76), sigma=3.0, lam=1.65, meff=0.2, dt=dt)
        f0 = lat.download_fields()
    f32 = {k: (v.astype(np.complex64).astype(np.complex128) if np.iscomplexobj(v)
               else v.astype(np.float32).astype(np.float64)) for k, v in f0.items()}
    with Lattice(N, precision="fp64") as lat:
        lat.upload_fields(f32)
        lat.step(dt, steps, save_uold=False)
        e64 = lat.bulk()[9]
    with _fp32(f32, N, reunitarize_every=16) as lat:
        lat.step(dt, steps, save_uold=False)
        e12, u12 = lat.bulk()[9], lat.unitarity()[0]
    assert abs(e12 - e64) <= 3e-4 * abs(e64), (e12, e64)
    assert u12 < 1e-5
