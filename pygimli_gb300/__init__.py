"""pygimli_gb300 -- GB300-native ERT (DC resistivity) forward operator and
Jacobian with pyGIMLi's ``ERTModelling`` method surface.

Host modules (numpy): mesh containers and generators (``mesh``), data
container and schemes (``data``), wavenumbers (``kwave``), model mapping
(``modelmap``).  Compute: ``ert.ERTModelling`` over libertgb.so
(hand-written sm_103a CUDA, C ABI in include/ertgb.h).
"""
from .data import DataContainerERT, createData, geometricFactors  # noqa: F401
from .mesh import Mesh, create_box_mesh_3d, create_para_mesh_2d  # noqa: F401

__all__ = ["DataContainerERT", "createData", "geometricFactors", "Mesh", "create_box_mesh_3d",
           "create_para_mesh_2d", "ERTModelling", "simulate"]


def __getattr__(name):
    if name in ("ERTModelling", "simulate"):
        from . import ert
        return getattr(ert, name)
    raise AttributeError(name)
