"""GB300-native engine for GravHopper's force-and-integrate path.

Import surface as the reference package (gravhopper/__init__.py:1-9):
``Simulation``, ``IC`` and ``grav`` (the ``jbgrav`` force functions).
"""
__version__ = "1.2.0+gb300.1"

from . import jbgrav as grav  # noqa: F401
from .gravhopper import (IC, DeviceForce, ExternalPackageException, GravHopperException,  # noqa: F401
                         ICException, Simulation, UninitializedSimulationException,
                         UnknownAlgorithmException)
