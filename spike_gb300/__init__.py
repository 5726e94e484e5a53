"""spike_gb300 - GB300-native clock-driven spiking-network step engine.

The step (LIF update + threshold + spike compaction, Poisson input, delayed
propagation, weight-dependent STDP) runs as hand-written sm_103a CUDA behind
the C ABI in include/spike_gb300.h; this package is the Python binding and the
model-building mirror used by the tests and the benchmark.
"""
from ._native import (SPK_CONN_ALL_TO_ALL, SPK_CONN_GAUSSIAN_SAMPLE, SPK_CONN_ONE_TO_ONE,  # noqa: F401
                      SPK_CONN_PAIRWISE, SPK_CONN_RANDOM, SPK_FIELD_INPUT_NEXT, SPK_FIELD_LAST_SPIKE,
                      SPK_FIELD_POST_TRACE, SPK_FIELD_PRE_TRACE, SPK_FIELD_RING, SPK_FIELD_SYN_TRACE,
                      SPK_FIELD_V, SPK_INPUT_NONE, SPK_INPUT_PATTERNED, SPK_INPUT_POISSON,
                      SPK_POP_INPUTS, SPK_POP_NEURONS, SPK_SYN_CONDUCTANCE, SPK_SYN_CURRENT,
                      SPK_SYN_VOLTAGE, SpikeError, lib)
from .model import (Batch, GenNetwork, LIFParams, Model, Net, Projection, Server, STDPParams,  # noqa: F401
                    SynapseParams, desc_arrays, schedule)

__all__ = ["Model", "Net", "Batch", "Server", "GenNetwork", "Projection", "LIFParams", "SynapseParams",
           "STDPParams", "schedule", "lib"]
