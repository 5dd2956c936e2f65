"""Configuration files through a device lattice: the text files a lattice writes equal the host
writer's (which reproduces the reference's files byte for byte, tests/test_checkpoint_text.py), and
a binary restart file reproduces every dynamical field bit for bit, so the evolution after a reload
is identical."""
import numpy as np
import pytest

from oracle import oracle as O
from soerenpragya3dglasma_gb300 import GlasmaError, Lattice, build
from soerenpragya3dglasma_gb300.checkpoint import read_text, write_text

pytestmark = pytest.mark.gpu

N = (6, 5, 7)
FIELDS = ("U", "UOld", "E", "Jp", "Jm", "JpStat", "JmStat")


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def test_lattice_text_files_equal_host_writer(tmp_path):
    f = O.random_fields(N, 91)
    mine = {k: tmp_path / ("dev_" + k + ".txt") for k in ("links", "efield", "currents")}
    host = {k: tmp_path / ("host_" + k + ".txt") for k in ("links", "efield", "currents")}
    with Lattice(N) as lat:
        lat.upload_fields(f)
        lat.save_text(**mine)
    write_text(N, f, **host)
    for k in mine:
        assert mine[k].read_bytes() == host[k].read_bytes(), k
    with Lattice(N) as lat:
        lat.load_text(**mine)
        got = {k: lat.download(k) for k in ("U", "E", "Jp", "Jm", "JpStat", "JmStat")}
    want = read_text(N, **host)
    for k in got:
        assert np.array_equal(got[k], want[k]), k


def test_binary_restart_is_bit_exact(tmp_path):
    f = O.random_fields(N, 92)
    path = tmp_path / "restart.bin"
    with Lattice(N) as a:
        a.upload_fields(f)
        a.step(0.1, 3)
        a.save_binary(path)
        before = {k: a.download(k) for k in FIELDS}
        a.step(0.1, 4)
        after_a = {k: a.download(k) for k in FIELDS}
    with Lattice(N) as b:
        b.load_binary(path)
        for k in FIELDS:
            assert np.array_equal(b.download(k), before[k]), k
        b.step(0.1, 4)
        for k in FIELDS:
            assert np.array_equal(b.download(k), after_a[k]), k


def test_binary_file_for_another_lattice_is_refused(tmp_path):
    path = tmp_path / "restart.bin"
    with Lattice(N) as a:
        a.upload_fields(O.random_fields(N, 93))
        a.save_binary(path)
    with Lattice((N[0], N[1], N[2] + 1)) as b:
        with pytest.raises(GlasmaError) as ei:
            b.load_binary(path)
        assert ei.value.status == 2  # GLASMA_ERR_BAD_SHAPE
    junk = tmp_path / "junk.bin"
    junk.write_bytes(b"not a configuration")
    with Lattice(N) as c:
        with pytest.raises(GlasmaError, match="not a binary configuration file"):
            c.load_binary(junk)
