"""Configuration files in the reference's text format, pinned on the reference's own writer and
loader (tests/golden/config_text.npz: IO::SaveConfiguration / SaveConfigurationJ output of seeded
fields and what IO::LoadConfiguration reads back).  Host-side only: no GPU."""
import os

import numpy as np
import pytest

from soerenpragya3dglasma_gb300 import GlasmaError, build
from soerenpragya3dglasma_gb300.checkpoint import read_text, write_text

CURRENTS = ("JpStat", "Jp", "JmStat", "Jm")


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


@pytest.fixture(scope="module")
def golden(golden_dir):
    return dict(np.load(os.path.join(golden_dir, "config_text.npz")))


def _fields(g):
    return {k[3:]: g[k] for k in g if k.startswith("in_")}


def _write_reference_files(g, tmp_path):
    paths = {}
    for name in ("links", "efield", "currents"):
        p = tmp_path / ("ref_" + name + ".txt")
        p.write_bytes(g["file_" + name].tobytes())
        paths[name] = p
    return paths


def test_writer_reproduces_the_reference_files_byte_for_byte(golden, tmp_path):
    N = tuple(int(v) for v in golden["cfg_N"])
    paths = {k: tmp_path / (k + ".txt") for k in ("links", "efield", "currents")}
    write_text(N, _fields(golden), **paths)
    for name, p in paths.items():
        assert p.read_bytes() == golden["file_" + name].tobytes(), name


def test_reader_matches_the_reference_loader(golden, tmp_path):
    N = tuple(int(v) for v in golden["cfg_N"])
    got = read_text(N, **_write_reference_files(golden, tmp_path))
    # links and E: the same text parsed by both sides, so the same doubles
    assert np.array_equal(got["U"], golden["loaded_U"])
    assert np.array_equal(got["E"], golden["loaded_E"])
    # currents: the reference's loader fills colours 0-2 only (its loop starts at the line's colour
    # and stops at 3); those agree, and colours 3-7 come from the file, which holds the inputs to
    # 15 significant digits
    for k in CURRENTS:
        assert np.array_equal(got[k][..., :3], golden["loaded_" + k][..., :3]), k
        assert np.all(golden["loaded_" + k][..., 3:] == 7.0), k  # the sentinel the reference left
        want = np.vectorize(lambda v: float("%.15g" % v))(golden["in_" + k])
        assert np.array_equal(got[k], want), k


def test_text_round_trip_keeps_fifteen_digits(golden, tmp_path):
    N = tuple(int(v) for v in golden["cfg_N"])
    f = _fields(golden)
    paths = {k: tmp_path / (k + ".txt") for k in ("links", "efield", "currents")}
    write_text(N, f, **paths)
    got = read_text(N, **paths)
    for k in ("U", "E") + CURRENTS:
        x = f[k].view(np.float64) if np.iscomplexobj(f[k]) else f[k]
        y = got[k].view(np.float64) if np.iscomplexobj(got[k]) else got[k]
        assert np.all(np.abs(y - x) <= 5e-15 * np.abs(x)), k


def test_malformed_files_return_a_status(golden, tmp_path):
    N = tuple(int(v) for v in golden["cfg_N"])
    paths = _write_reference_files(golden, tmp_path)
    lines = paths["links"].read_text().splitlines(keepends=True)
    short = tmp_path / "short.txt"
    short.write_text("".join(lines[:-1]))
    with pytest.raises(GlasmaError, match="file ends before all links"):
        read_text(N, links=short)
    swapped = tmp_path / "swapped.txt"
    swapped.write_text("".join([lines[1], lines[0]] + lines[2:]))
    with pytest.raises(GlasmaError, match="swapped.txt:1: expected link 0 0 -1 0"):
        read_text(N, links=swapped)
    with pytest.raises(GlasmaError, match="cannot open"):
        read_text(N, efield=tmp_path / "missing.txt")
    with pytest.raises(GlasmaError, match="expected field 3 0 -1 0"):  # a file for another lattice shape
        read_text((N[0] + 1, N[1], N[2]), efield=paths["efield"])
