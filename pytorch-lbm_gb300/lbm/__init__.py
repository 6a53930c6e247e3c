"""GB300-native Allen-Cahn phase-field LBM with the reference's Python surface.

Modules keep the reference's names (pytorch-lbm ``lbm/``): ``fe_config``
(FEConfig), ``fe_ac_solver`` (AllenCahnSolver), ``fe_droplet`` (initial
droplets), ``fe_measure`` (diagnostics), ``lattice`` (D3Q19).
"""
from .fe_config import FEConfig  # noqa: F401
