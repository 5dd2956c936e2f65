"""The C++ drop-in (include/glasma_gb300_reference_api.hpp): a driver written against the
reference's namespaces compiles against the header and reproduces the oracle's evolution."""
import os
import subprocess

import numpy as np
import pytest

from oracle import oracle as O
from soerenpragya3dglasma_gb300 import build
from soerenpragya3dglasma_gb300.checkpoint import read_text

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "dropin_evolve.cpp")


def compile_driver(tmp_path):
    lib = build.build()
    exe = str(tmp_path / "dropin_evolve")
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
           "-L", os.path.dirname(lib), "-lglasma_gb300", "-Wl,-rpath," + os.path.dirname(lib)]
    subprocess.check_call(cmd)
    return exe


def test_dropin_header_compiles(tmp_path):
    compile_driver(tmp_path)


@pytest.mark.gpu
def test_dropin_driver_matches_oracle(tmp_path, oracle):
    exe = compile_driver(tmp_path)
    N, dt, steps = (6, 6, 10), 0.125, 4
    f = O.random_fields(N, 808)
    for k in ("U", "E", "Jp", "Jm", "JpStat", "JmStat"):
        f[k].tofile(str(tmp_path / ("in.%s.bin" % k)))
    r = subprocess.run([exe, str(N[0]), str(N[1]), str(N[2]), repr(dt), str(steps), str(tmp_path / "in"),
                        str(tmp_path / "out")], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    vals = {l.split()[0]: [float(x) for x in l.split()[1:]] for l in r.stdout.splitlines()}
    ref = O.copy_fields(f)
    oracle.update(ref, N, (1.0, 1.0, 1.0), dt, steps)
    for k in O.FIELD_NAMES:
        got = np.fromfile(str(tmp_path / ("out.%s.bin" % k)), dtype=ref[k].dtype).reshape(ref[k].shape)
        assert np.max(np.abs(got - ref[k])) / np.max(np.abs(ref[k])) < 1e-12, k
    bulk = oracle.bulk(ref, N, (1.0, 1.0, 1.0))
    assert abs(vals["T00"][0] - bulk[9]) / abs(bulk[9]) < 1e-12
    assert np.allclose(vals["GAUSS"], oracle.gauss(ref, N, (1.0, 1.0, 1.0)), rtol=1e-12)
    assert abs(vals["TIME"][0] - steps * dt) < 1e-12
    # the reference's text configuration files, written through IO::SaveConfiguration(J)
    txt = read_text(N, links=tmp_path / "out.UID0.txt", efield=tmp_path / "out.EID0.txt",
                    currents=tmp_path / "out.JID0.txt")
    for k in ("U", "E", "Jp", "Jm", "JpStat", "JmStat"):
        got = np.fromfile(str(tmp_path / ("out.%s.bin" % k)), dtype=ref[k].dtype).reshape(ref[k].shape)
        x = got.view(np.float64) if np.iscomplexobj(got) else got
        y = txt[k].view(np.float64) if np.iscomplexobj(txt[k]) else txt[k]
        assert np.all(np.abs(y - x) <= 6e-15 * np.abs(x)), k  # 15 significant digits, then a parse
