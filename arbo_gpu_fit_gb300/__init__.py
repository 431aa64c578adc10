"""GB300-native (sm_103a) per-time-step dengue agent simulation behind the reference's host API.

The compute path is the native library ``_lib/libarbo_gb300.so`` (CUDA kernels + C-ABI,
include/arbo.h); this package is the host-side mirror of the reference's interface.
"""
from .simulation import (ArchitectureParam, Batch, IOParam, Network, Parameter, Simulation, SimulationParam,
                         calc_cumulative_com_size, community_sizes, create_network, simulation)

__all__ = ["ArchitectureParam", "Batch", "IOParam", "Network", "Parameter", "Simulation", "SimulationParam",
           "calc_cumulative_com_size", "community_sizes", "create_network", "simulation"]
