"""GB300-native real-time SU(3) glasma path: leapfrog, observables and Coulomb gauge
fixing as hand-written sm_103a kernels behind a C ABI (include/glasma_gb300.h).

    from soerenpragya3dglasma_gb300 import Lattice
    lat = Lattice((Nx, Ny, Nz), a=(1, 1, 1), precision="fp64")
    lat.upload("U", U); ...; lat.step(dt, nsteps); lat.bulk()

`reference_api` mirrors the reference's own namespaces (Dynamics::SUNc::Update,
Observables::Bulk, ...) over the same handle.
"""
from ._lib import GlasmaError, load  # noqa: F401
from .batch import Batch  # noqa: F401
from .lattice import DYNAMICAL_FIELDS, Lattice, empty_field, field_shape, glauber_sample, tmd_default_params  # noqa: F401

__all__ = ["Lattice", "Batch", "GlasmaError", "load", "field_shape", "empty_field", "DYNAMICAL_FIELDS",
           "glauber_sample", "tmd_default_params"]
