"""GB300 (sm_103a) implementation of the per-tet implicit-arrangement path of
Robust-Implicit-Surface-Networks: sampling, sign filter, per-tet cut and mesh extraction on the
GPU behind the C ABI of include/ria.h.

The directory name contains hyphens; import it with
    importlib.import_module("robust-implicit-surface-networks_gb300")
"""
from . import functions  # noqa: F401
from ._lib import RiaError, declared_functions, load  # noqa: F401
from .api import (BatchMesh, Mesh, Server, compute_arrangement_batch, grid_batch, compute_material_interface_batch, device_count,  # noqa: F401
                  grid_implicit_arrangement, grid_material_interface, implicit_arrangement, material_interface,
                  sample_functions, get_tuning, set_tuning, autotune)


def build(verbose: bool = False) -> str:
    from .build_lib import build as _build

    return _build(verbose=verbose)
