"""Size-independent properties at the production workload's size, 128x128x512 (8.4 M sites), on seeded
synthetic fields generated on the device.  The oracle would take hours here, so each test checks a
property that holds exactly in exact arithmetic, with a rounding-level tolerance:
  * the plaquette method and the staple (two-pass) method, two different summations of the same
    force, give the same fields;
  * the one-pass and two-pass methods give bit-identical fields;
  * with zero colour currents the Gauss law G(x) is conserved by the leapfrog in every slice but
    z = 0 (the oracle restatement shows the same: interior slices to 1e-16, slice 0 not, by the
    reference's open-boundary convention);
  * 12-real FP32 links follow 18-real FP32 links, and FP32 follows FP64 in the energy."""
import numpy as np
import pytest

from soerenpragya3dglasma_gb300 import Lattice, build

pytestmark = pytest.mark.gpu

N = (128, 128, 512)
DT = 0.125
SEED = 1002


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def _lattice(precision="fp64", method="plaquette", reals=18, j_amp=0.02, **kw):
    lat = Lattice(N, precision=precision, **kw)
    lat.set_step_method(method)
    if reals != 18:
        lat.link_reals = reals
    lat.fill_synthetic(SEED, 0.3, 0.1, j_amp)
    return lat


def _device_fields(lat, names=("U", "E", "Jp", "JpStat")):
    """The fields in the host layout, in device memory (torch), without a trip through the host."""
    torch = pytest.importorskip("torch")
    out = {}
    for k in names:
        t = torch.empty(lat.field_doubles(k), dtype=torch.float64, device="cuda")
        lat.download_device(k, t.data_ptr())
        out[k] = t
    torch.cuda.synchronize()
    return out


def _rel(a, b):
    return float((a - b).abs().max() / b.abs().max())


def test_plaquette_method_equals_staple_form():
    with _lattice(method="plaquette") as a, _lattice(method="two_pass") as b:
        a.step(DT, 3, save_uold=False)
        b.step(DT, 3, save_uold=False)
        assert a.last_step_method == "plaquette" and b.last_step_method == "two_pass"
        fa, fb = _device_fields(a), _device_fields(b)
        for k in fa:
            assert _rel(fa[k], fb[k]) < 1e-12, k
        assert np.allclose(a.bulk(), b.bulk(), rtol=1e-12, atol=1e-12)


def test_one_pass_equals_two_pass_bit_exact():
    torch = pytest.importorskip("torch")
    with _lattice(method="one_pass") as a, _lattice(method="two_pass") as b:
        a.step(DT, 2, save_uold=True)
        b.step(DT, 2, save_uold=True)
        fa, fb = _device_fields(a, ("U", "UOld", "E", "Jp", "Jm", "JpStat", "JmStat")), \
            _device_fields(b, ("U", "UOld", "E", "Jp", "Jm", "JpStat", "JmStat"))
        for k in fa:
            assert torch.equal(fa[k], fb[k]), k


@pytest.mark.parametrize("precision,method,tol", [("fp64", "plaquette", 1e-11), ("fp64", "two_pass", 1e-11),
                                                  ("fp32", "plaquette", 2e-5)])
def test_gauss_law_conserved_in_the_interior_slices(precision, method, tol):
    with _lattice(precision=precision, method=method, j_amp=0.0) as lat:
        _, _, p0 = lat.gauss(sync_first=True, profile=True)
        lat.step(DT, 4, save_uold=False)
        _, _, p1 = lat.gauss(sync_first=True, profile=True)
    p0, p1 = np.asarray(p0), np.asarray(p1)
    assert p0.shape == (N[2],)
    assert np.max(np.abs(p1[1:] - p0[1:]) / p0[1:]) < tol
    if precision == "fp64":  # slice 0 is not conserved (open boundary), as in the oracle
        assert abs(p1[0] - p0[0]) > 1e-6 * p0[0]


def test_fp32_links12_and_fp64_agree_on_the_energy():
    with _lattice(precision="fp64") as d:
        d.step(DT, 16, save_uold=False)
        e64 = d.bulk()[9]
    out = {}
    for reals in (18, 12):
        with _lattice(precision="fp32", reals=reals, reunitarize_every=16) as f:
            f.step(DT, 16, save_uold=False)
            out[reals] = (f.bulk()[9], _device_fields(f, ("U", "E")), f.unitarity()[0])
    for reals in (18, 12):
        assert abs(out[reals][0] - e64) < 1e-6 * abs(e64), reals
        assert out[reals][2] < 1e-5, reals
    for k in ("U", "E"):
        assert _rel(out[12][1][k], out[18][1][k]) < 1e-4, k
