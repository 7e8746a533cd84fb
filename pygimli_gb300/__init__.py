"""pygimli_gb300 -- GB300-native ERT (DC resistivity) forward operator and
Jacobian with pyGIMLi's ``ERTModelling`` method surface.

Host modules (numpy): mesh containers and generators (``mesh``), data
container and schemes (``data``), the reference's file formats (``fileio``:
unified data files, binary meshes, VTK export), wavenumbers (``kwave``),
model mapping (``modelmap``).  Compute: ``ert.ERTModelling`` over libertgb.so
(hand-written sm_103a CUDA, C ABI in include/ertgb.h).
"""
from .data import DataContainerERT, createData, geometricFactors  # noqa: F401
from .mesh import Mesh, create_box_mesh_3d, create_para_mesh_2d  # noqa: F401

__all__ = ["DataContainerERT", "createData", "geometricFactors", "Mesh", "create_box_mesh_3d",
           "create_para_mesh_2d", "ERTModelling", "simulate", "createGeometricFactors", "load"]


def load(fileName, **kwargs):
    """A binary mesh ('.bms') as ``Mesh``, anything else as a unified data
    file in a ``DataContainerERT`` (the two file kinds ``pg.load`` and
    ``pg.physics.ert.load`` read with the reference's own loaders)."""
    import os
    if os.fspath(fileName).endswith(".bms"):
        return Mesh.load(fileName)
    return DataContainerERT(fileName, **kwargs)


def __getattr__(name):
    if name in ("ERTModelling", "simulate", "createGeometricFactors"):
        from . import ert
        return getattr(ert, name)
    raise AttributeError(name)
