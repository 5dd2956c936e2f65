"""Batched multi-event stepping (one launch per kernel over all events, CUDA-graph replay), with the
plaquette and the two-pass method: bit-identical to stepping each event alone with the same method,
and the FP64 batch matches the oracle."""
import numpy as np
import pytest

from oracle import oracle as O
from soerenpragya3dglasma_gb300 import Batch, Lattice, build

pytestmark = pytest.mark.gpu

SHAPES = [(6, 5, 8), (12, 8, 20), (4, 4, 6), (9, 7, 11)]


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_batch_equals_individual_events(precision):
    fields = [O.random_fields(N, 300 + i) for i, N in enumerate(SHAPES)]
    dt, steps = 0.1, 37  # crosses two 16-step graph blocks plus single steps
    with Batch(SHAPES, precision=precision, reunitarize_every=16) as b:
        b.set_step_method("two_pass")
        tiles = b.autotune(dt)
        assert len(tiles) == len(SHAPES)
        for ev, f in zip(b.events, fields):
            ev.upload_fields(f)
        b.step(dt, steps, use_graph=True)
        got = [ev.download_fields(("U", "E", "Jp", "Jm", "JpStat", "JmStat")) for ev in b.events]
        energies = b.energy()
    for i, (N, f) in enumerate(zip(SHAPES, fields)):
        with Lattice(N, precision=precision, reunitarize_every=16) as lat:
            lat.set_step_method("two_pass")  # the batch's two-pass method: the staple kernels
            lat.set_tile(tiles[i])
            lat.upload_fields(f)
            lat.step(dt, steps, save_uold=False)
            ref = lat.download_fields(("U", "E", "Jp", "Jm", "JpStat", "JmStat"))
            assert energies[i] == lat.bulk()[9], i
        for k in ref:
            assert np.array_equal(got[i][k], ref[k]), (i, k)


@pytest.mark.parametrize("mode", ["tile_grid", "persistent"])
def test_batch_links12_equals_individual_events(mode):
    """12-real links in the batched kernels: bit-identical to each event stepped alone with 12-real
    links, in both launch modes; full links after the call."""
    fields = [O.random_fields(N, 340 + i) for i, N in enumerate(SHAPES)]
    dt, steps = 0.1, 37
    with Batch(SHAPES, precision="fp32", reunitarize_every=16) as b:
        b.set_step_method("two_pass")
        b.set_launch(mode)
        b.set_link_reals(12)
        tiles = b.autotune(dt)
        for ev, f in zip(b.events, fields):
            ev.upload_fields(f)
        b.step(dt, steps, use_graph=True)
        got = [ev.download_fields(("U", "E", "Jp", "Jm", "JpStat", "JmStat")) for ev in b.events]
        umax = max(ev.unitarity()[0] for ev in b.events)
    assert umax < 1e-5
    for i, (N, f) in enumerate(zip(SHAPES, fields)):
        with Lattice(N, precision="fp32", reunitarize_every=16) as lat:
            lat.set_step_method("two_pass")
            lat.link_reals = 12
            lat.set_tile(tiles[i])
            lat.upload_fields(f)
            lat.step(dt, steps, save_uold=False)
            ref = lat.download_fields(("U", "E", "Jp", "Jm", "JpStat", "JmStat"))
        for k in ref:
            assert np.array_equal(got[i][k], ref[k]), (i, k)
    with Batch(SHAPES, precision="fp64") as b:
        with pytest.raises(Exception):
            b.set_link_reals(12)


@pytest.mark.parametrize("precision,reals,mode", [("fp64", 18, "tile_grid"), ("fp64", 18, "persistent"),
                                                   ("fp32", 18, "tile_grid"), ("fp32", 12, "persistent")])
def test_batch_plaquette_equals_individual_events(precision, reals, mode):
    """The plaquette method over the batch: each event's fields bit-identical to the event stepped
    alone with the plaquette method (graph blocks, reunitarisation and single steps crossed)."""
    fields = [O.random_fields(N, 360 + i) for i, N in enumerate(SHAPES)]
    dt, steps = 0.1, 37
    with Batch(SHAPES, precision=precision, reunitarize_every=16) as b:
        assert b.step_method() == "plaquette"  # the default
        b.set_step_method("two_pass")
        assert b.step_method() == "two_pass"
        b.set_step_method("plaquette")
        b.set_launch(mode)
        if reals == 12:
            b.set_link_reals(12)
        for ev, f in zip(b.events, fields):
            ev.upload_fields(f)
        b.step(dt, steps, use_graph=True)
        assert b.step_method() == "plaquette"
        got = [ev.download_fields(("U", "E", "Jp", "Jm", "JpStat", "JmStat")) for ev in b.events]
        with pytest.raises(Exception):
            b.set_step_method("one_pass")
    for i, (N, f) in enumerate(zip(SHAPES, fields)):
        with Lattice(N, precision=precision, reunitarize_every=16) as lat:
            lat.set_step_method("plaquette")
            if reals == 12:
                lat.link_reals = 12
            lat.upload_fields(f)
            lat.step(dt, steps, save_uold=False)
            ref = lat.download_fields(("U", "E", "Jp", "Jm", "JpStat", "JmStat"))
        for k in ref:
            assert np.array_equal(got[i][k], ref[k]), (i, k)


def test_batch_plaquette_fp64_matches_oracle(oracle):
    fields = [O.random_fields(N, 410 + i) for i, N in enumerate(SHAPES)]
    dt, steps = 0.125, 5
    with Batch(SHAPES, precision="fp64") as b:
        for ev, f in zip(b.events, fields):
            ev.upload_fields(f)
        b.step(dt, steps, use_graph=False)
        got = [ev.download_fields() for ev in b.events]
    for N, f, g in zip(SHAPES, fields, got):
        ref = O.copy_fields(f)
        oracle.update(ref, N, (1.0, 1.0, 1.0), dt, steps, save_uold=False)
        for k in ("U", "E", "Jp", "Jm", "JpStat", "JmStat"):
            assert np.max(np.abs(g[k] - ref[k])) / np.max(np.abs(ref[k])) < 1e-12, k


def test_batch_launch_modes_agree():
    """One block per tile and the persistent grid run the same per-site arithmetic."""
    fields = [O.random_fields(N, 330 + i) for i, N in enumerate(SHAPES)]
    out = []
    for mode in ("tile_grid", "persistent"):
        with Batch(SHAPES, precision="fp32", reunitarize_every=16) as b:
            b.set_launch(mode)
            for ev, f in zip(b.events, fields):
                ev.upload_fields(f)
            b.step(0.1, 20, use_graph=True)
            out.append([ev.download_fields(("U", "E", "Jp", "JmStat")) for ev in b.events])
    for a, c in zip(out[0], out[1]):
        for k in a:
            assert np.array_equal(a[k], c[k]), k


def test_batch_after_events_stepped_alone():
    """Stepping an event on its own (one-pass: its buffers swap) between batched steps: the batch
    rebuilds its event table and the result equals stepping every event alone."""
    fields = [O.random_fields(N, 350 + i) for i, N in enumerate(SHAPES)]
    dt = 0.1
    with Batch(SHAPES, precision="fp64") as b:
        b.set_step_method("two_pass")
        for ev, f in zip(b.events, fields):
            ev.upload_fields(f)
        b.step(dt, 2, use_graph=False)
        for i in (1, 2):
            b.events[i].set_step_method("one_pass")
            b.events[i].step(dt, 1, save_uold=False)
        b.step(dt, 3, use_graph=False)
        got = [ev.download_fields(("U", "E", "Jp", "Jm", "JpStat", "JmStat")) for ev in b.events]
    for i, (N, f) in enumerate(zip(SHAPES, fields)):
        with Lattice(N) as lat:
            lat.set_step_method("two_pass")
            lat.upload_fields(f)
            lat.step(dt, 2, save_uold=False)
            if i in (1, 2):
                lat.step(dt, 1, save_uold=False)
            lat.step(dt, 3, save_uold=False)
            ref = lat.download_fields(("U", "E", "Jp", "Jm", "JpStat", "JmStat"))
        for k in ref:
            assert np.array_equal(got[i][k], ref[k]), (i, k)


def test_batch_fp64_matches_oracle(oracle):
    fields = [O.random_fields(N, 400 + i) for i, N in enumerate(SHAPES)]
    dt, steps = 0.125, 5
    with Batch(SHAPES, precision="fp64") as b:
        b.set_step_method("two_pass")
        for ev, f in zip(b.events, fields):
            ev.upload_fields(f)
        b.step(dt, steps, use_graph=False)
        got = [ev.download_fields() for ev in b.events]
    for N, f, g in zip(SHAPES, fields, got):
        ref = O.copy_fields(f)
        oracle.update(ref, N, (1.0, 1.0, 1.0), dt, steps, save_uold=False)
        for k in ("U", "E", "Jp", "Jm", "JpStat", "JmStat"):
            assert np.max(np.abs(g[k] - ref[k])) / np.max(np.abs(ref[k])) < 1e-12, k


def test_fill_synthetic_is_seeded_and_unitary():
    N = (8, 6, 10)
    with Lattice(N) as a, Lattice(N) as b:
        a.fill_synthetic(7, link_amp=0.3, e_amp=0.1, j_amp=0.02)
        b.fill_synthetic(7, link_amp=0.3, e_amp=0.1, j_amp=0.02)
        fa, fb = a.download_fields(), b.download_fields()
        assert a.unitarity()[0] < 1e-13
    for k in ("U", "E", "Jp", "JmStat"):
        assert np.array_equal(fa[k], fb[k]), k
    E = fa["E"][1:-1]
    assert abs(E.mean()) < 0.01 and abs(E.std() - 0.1) < 0.01
    assert np.array_equal(fa["E"][0], fa["E"][1]) and np.array_equal(fa["U"][-1], fa["U"][-2])
