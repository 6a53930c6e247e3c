"""GB300-native Allen-Cahn phase-field LBM with the reference's Python surface.

Modules keep the reference's names (pytorch-lbm ``lbm/``): ``fe_config``
(FEConfig), ``fe_ac_solver`` (AllenCahnSolver), ``fe_droplet`` (initial
droplets), ``fe_measure`` (diagnostics), ``lattice`` (D2Q9, D3Q19); the
package exports the same names as the reference's (lbm/__init__.py).
"""
from .fe_ac_solver import AllenCahnSolver  # noqa: F401
from .fe_config import FEConfig  # noqa: F401
from .lattice import D2Q9, D3Q19  # noqa: F401
