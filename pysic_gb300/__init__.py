"""pysic_gb300 -- the Pysic energy/force API on a GB300-native engine.

Drop-in for the reference package ``pysic`` (pysic/__init__.py:1-17): the same
classes and descriptor queries, with energies, forces, electronegativities,
neighbour lists and charge relaxation computed by hand-written sm_103a CUDA
kernels behind a C ABI (include/pysic_gb300.h).  ``import pysic_gb300 as
pysic`` is the intended use.
"""
from .atoms import Atoms
from .calculator import FastNeighborList, Pysic
from .comb import CombPotential
from .core import *  # noqa: F401,F403  descriptor queries of pysic.core
from .error import *  # noqa: F401,F403
from .interactions import (BondOrderParameters, CompoundPotential, Coordinator, CoulombSummation, Potential,
                           ProductPotential, SuttonChenPotential, estimate_ewald_parameters)
from .md import VelocityVerlet
from .relaxation import ChargeRelaxation

__version__ = "0.1.0"

__all__ = ["Atoms", "Pysic", "VelocityVerlet", "FastNeighborList", "Potential", "ProductPotential", "BondOrderParameters", "Coordinator",
           "CoulombSummation", "ChargeRelaxation", "estimate_ewald_parameters", "CompoundPotential",
           "SuttonChenPotential", "CombPotential"]
