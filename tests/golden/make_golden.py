"""Generate the golden fixtures in this directory from the reference itself.

The reference's own SU(3) code path is compiled from its unmodified sources by
``oracle/build.py`` (``oracle/_ref/libglasma_ref.so``; only possible where the
reference checkout exists) and run on small seeded inputs.  Each reference run
happens in a child process: the reference keeps its fields in global singletons
and calls exit() on numerical failure.

    python tests/golden/make_golden.py

Fixtures (npz, float64/complex128, reference host layout with ghost slices):
  leapfrog_random.npz   4x4x6 lattice, anisotropic spacing, seeded hot links:
                        initial state, state after 1 and 10 steps of
                        Dynamics::SUNc::Update, observables at each point
  coulomb_mild.npz      4x4x6 lattice, weak field in a random gauge: 4 Fourier-
                        accelerated iterations (log, G, gauge-fixed U and E)
  expi.npz              MatrixIExp known answers
  mv_collision.npz      MV collision initial state on 4x4x16 (injected Gaussian
                        charges), observables at t=0 and after 8 steps
"""
import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

LEAPFROG = dict(N=(4, 4, 6), a=(1.0, 0.9, 0.7), dt=0.1, seed=1234)
COULOMB = dict(N=(4, 4, 6), a=(1.0, 1.0, 1.0), alpha=0.5, iters=4, seed=5)
MV = dict(N=(4, 4, 16), a=(1.0, 1.0, 1.0), dt=0.125, qs=0.5, sigma=2.0, lam=1.65, meff=0.2, seed=1001, steps=8)


def _observables(ref):
    out = {}
    out["bulk"] = ref.bulk()
    out["gauss"] = np.array(ref.gauss())
    out["gauss_profile"] = ref.gauss_profile()
    out["unitarity"] = np.array(ref.unitarity())
    out["emt"] = ref.emt_map()
    return out


def leapfrog_case(q):
    c = LEAPFROG
    f0 = O.random_fields(c["N"], c["seed"])
    ref = O.Reference(c["N"], c["a"])
    ref.set_fields(f0)
    res = {"init_" + k: v for k, v in f0.items()}
    for tag, nsteps in (("s1", 1), ("s10", 9)):
        ref.update(nsteps, c["dt"])
        for k, v in ref.get_fields().items():
            res[tag + "_" + k] = v
        for k, v in _observables(ref).items():
            res[tag + "_" + k] = v
    q.put(res)


def mild_gauge_config(N, seed, eps=0.02, om=0.2):
    """Weak random field V in a random gauge Om, top z-links set to the identity."""
    rng = np.random.default_rng(seed)
    Nx, Ny, Nz = N
    V = O.expi_batched(eps, rng.standard_normal((Nz + 2, Ny, Nx, 3, 8)))
    Om = O.expi_batched(om, rng.standard_normal((Nz + 2, Ny, Nx, 8)))
    U = np.empty_like(V)
    for mu in range(3):
        if mu < 2:
            Omf = np.roll(Om[1:-1], -1, axis=2 - mu)
        else:
            Omf = np.concatenate([Om[2:-1], Om[-2:-1]], axis=0)
        U[1:-1, :, :, mu] = np.einsum("...ij,...jk,...lk->...il", Om[1:-1], V[1:-1, :, :, mu], Omf.conj())
    U[-2, :, :, 2] = np.eye(3)
    f = O.random_fields(N, seed + 1)
    f["U"] = O.matrices_to_links(U)
    O.sync_ghosts(f["U"])
    return f


def coulomb_case(q):
    c = COULOMB
    f = mild_gauge_config(c["N"], c["seed"])
    ref = O.Reference(c["N"], c["a"])
    ref.set_fields(f)
    log = ref.coulomb_fix(c["alpha"], c["iters"])
    res = {"U": f["U"], "E": f["E"], "log": log, "G": ref.get("G"), "UG": ref.get("UG"), "EG": ref.get("EG")}
    q.put(res)


def expi_case(q):
    ref = O.Reference((2, 2, 2), (1.0, 1.0, 1.0))
    rng = np.random.default_rng(7)
    cs = np.array([1e-9, 1e-5, 0.01, 0.3, 1.0, -1.7, 2.5, 6.0])
    al = rng.standard_normal((len(cs), 8))
    al[0] = 0.0
    al[1] = [0, 0, 1.0, 0, 0, 0, 0, 0]  # degenerate eigenvalues (lambda_3 direction)
    al[2] = [0, 0, 0, 0, 0, 0, 0, 1.0]  # degenerate eigenvalues (lambda_8 direction)
    out = np.array([ref.expi(c, a) for c, a in zip(cs, al)])
    q.put({"c": cs, "alpha": al, "expi": out})


def mv_gaussians(N, seed, two_nuclei=True):
    rng = np.random.Generator(np.random.PCG64(seed))
    Nx, Ny, _ = N
    n = 8 * Nx * Ny * (2 if two_nuclei else 1)
    return rng.standard_normal(n)


def mv_case(q):
    c = MV
    N = c["N"]
    g = mv_gaussians(N, c["seed"])
    ref = O.Reference(N, c["a"])
    Nz = N[2]
    cl, cr = Nz // 2 - 4, Nz // 2 + 4
    ref.mv_init(g, c["dt"], c["qs"], c["qs"], cl, cr, c["sigma"], c["lam"], c["meff"])
    res = {"gauss_in": g, "center_left": cl, "center_right": cr}
    for k, v in ref.get_fields().items():
        res["init_" + k] = v
    for k, v in _observables(ref).items():
        res["t0_" + k] = v
    ref.update(c["steps"], c["dt"])
    for k, v in _observables(ref).items():
        res["t8_" + k] = v
    q.put(res)


def run(fn):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    p = ctx.Process(target=fn, args=(q,))
    p.start()
    res = q.get(timeout=600)
    p.join()
    return res


def main():
    from oracle import build

    if build.build_reference() is None:
        raise SystemExit("reference sources not found; fixtures can only be generated where they exist")
    r = run(leapfrog_case)
    np.savez_compressed(os.path.join(HERE, "leapfrog_random.npz"), **r, **{"cfg_" + k: np.array(v) for k, v in LEAPFROG.items()})
    r = run(coulomb_case)
    np.savez_compressed(os.path.join(HERE, "coulomb_mild.npz"), **r, **{"cfg_" + k: np.array(v) for k, v in COULOMB.items()})
    r = run(expi_case)
    np.savez_compressed(os.path.join(HERE, "expi.npz"), **r)
    r = run(mv_case)
    np.savez_compressed(os.path.join(HERE, "mv_collision.npz"), **r, **{"cfg_" + k: np.array(v) for k, v in MV.items()})
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
