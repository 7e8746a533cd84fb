"""Generate the fixtures of a Jacobian requested before any response, by
running the reference's own C++ (oracle/_ref/libgimli_ref.so, built by
``make -C oracle``) through oracle/ref_driver.py on a fresh operator:

    python tests/golden/make_jacobian_first_golden.py

The reference then computes the sub-potentials itself
(DCMultiElectrodeModelling::prepareJacobianT_, core/src/bert/
dcfemmodelling.cpp:1262-1301): analytically for a homogeneous model (scaled
by its value), by a response to the model otherwise.  Meshes, schemes and
the heterogeneous model are those of the ert2d_small / ert3d_small fixtures.

  jacobian_first_small.npz: J_hom_2d, J_het_2d (2.5-D), J_hom_3d, J_het_3d (3-D)
  and the homogeneous value rho_hom.

Run from the repository root.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle.ref_driver import RefModelling  # noqa: E402
from pygimli_gb300.mesh import Mesh  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
RHO_HOM = 73.0


def fresh_jacobian(z, model):
    mesh = Mesh(int(z["dim"]), z["nodes"], z["cells"], z["cell_markers"], z["node_markers"], z["boundaries"],
                z["boundary_markers"], z["boundary_cells"])
    R = RefModelling(mesh, z["sensors"], z["abmn"], z["kfac"])
    R.set_kw(z["k"], z["w"])
    J = R.jacobian(model)
    R.close()
    return J


def main():
    out = {"rho_hom": RHO_HOM}
    for tag, name in (("2d", "ert2d_small"), ("3d", "ert3d_small")):
        z = np.load(os.path.join(OUT, name + ".npz"))
        C = len(z["cells"])
        out["J_hom_" + tag] = fresh_jacobian(z, np.full(C, RHO_HOM))
        out["J_het_" + tag] = fresh_jacobian(z, z["rho"])
        print(name, out["J_hom_" + tag].shape)
    np.savez_compressed(os.path.join(OUT, "jacobian_first_small.npz"), **out)


if __name__ == "__main__":
    main()
