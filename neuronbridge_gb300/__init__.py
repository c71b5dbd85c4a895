"""neuronbridge_gb300 -- GB300-native step engine for NeuronBridge networks.

The public names mirror the reference's ``neuronbridge`` package (Network,
NeuronLayer, Connection, LearningRule, SimulationConfig, Simulation and the
typed-parameter helpers) so network-building code written for the reference
runs unchanged; the work is done by hand-written sm_103a CUDA kernels behind
the C ABI in ``include/nbg.h``.
"""
from ._lib import NbgError, load
from .model import (CATALOG, Connection, LearningRule, NativeParameter, Network, NetworkDescription, NeuronLayer,
                    SimulationConfig, float32, float32_list, float64, int32, resolve_model)
from .simulation import Simulation
from . import nbnet
from .debug_monitor import DebugMonitorConfig, DebugMonitorResult, open_debug_monitor
from .nbnet import StreamingBuildOptions

__all__ = [
    "CATALOG", "Connection", "LearningRule", "NativeParameter", "NbgError", "Network", "NetworkDescription",
    "NeuronLayer", "Simulation", "SimulationConfig", "float32", "float32_list", "float64", "int32", "load",
    "resolve_model", "nbnet", "StreamingBuildOptions", "DebugMonitorConfig", "DebugMonitorResult",
    "open_debug_monitor",
]
