"""bluetangle_gpu — host-side mirror of BlueTangle.jl's noisy-circuit API over libbtgpu.

The hot path (gates, channels, measurement, sampling, observables) runs in the
sm_103a CUDA library libbtgpu.so through its C ABI (include/btgpu.h); this
package only builds the reference's op descriptors and small host tables and
calls the library.  The first engine call (a Context, a state, a plan) loads the
library and raises ImportError if it is absent: there is no CPU path.  Importing
the package alone maps no native code, so the pure-host parts (gate tables, op
descriptors, circuit generators) serve tools that must not load it.
"""
from ._lib import BTError, lib
from .engine import (Context, GPUDensity, GPUState, Measurement, Plan, plan_from_ops, apply, apply_channel, apply_matrix, apply_noise,
                     born_measure_Z, channel_probs, correlation, expect, fidelity, measure, partial_trace,
                     pauli_masks, rho_from, run, sample, sample_exact, state_from, to_rho, to_state, zero_rho,
                     zero_state)
from .circuit import (Circuit, Options, Z3, Z3_s, compile, fidelity_dm, get_stats, measure, minus_state,
                      neel_state01, neel_state10, neel_state_s, one_state, plus_state, product_state,
                      random_product_state, random_state)
from .gates import gate, gates
from .noise import NoiseModel, Noise1, Noise2, QuantumChannel, apply_twirl, noise_model
from .ops import Op, OpQC, ifOp

__all__ = ["BTError", "Context", "Plan", "plan_from_ops", "GPUState", "GPUDensity", "Measurement", "apply", "apply_channel", "apply_matrix",
           "apply_noise", "born_measure_Z", "channel_probs", "correlation", "expect", "fidelity", "measure",
           "partial_trace", "pauli_masks", "rho_from", "run", "sample", "sample_exact", "state_from", "to_rho",
           "to_state", "zero_rho", "zero_state", "gate", "gates", "NoiseModel", "Noise1", "Noise2",
           "QuantumChannel", "apply_twirl", "noise_model", "Op", "OpQC", "ifOp", "Circuit", "Options", "compile",
           "get_stats", "product_state", "neel_state01", "neel_state10", "neel_state_s", "Z3", "Z3_s", "one_state",
           "plus_state", "minus_state", "random_product_state", "random_state", "fidelity_dm"]
