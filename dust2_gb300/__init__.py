"""GPU engine for dust2's data-parallel hot path, with a Python mirror of
dust2's R verbs.  The engine itself is the CUDA library built from
csrc/ (C ABI: include/dust2_gb300.h)."""

from ._lib import DustError, device_count
from .interface import (
    DustLikelihood, DustServer, DustSystem, DustUnfilter, Generator,
    dust_filter_create,
    dust_filter_data, dust_likelihood_last_gradient,
    dust_likelihood_last_state, dust_likelihood_rng_state,
    dust_likelihood_last_snapshots, dust_likelihood_last_trajectories,
    dust_likelihood_run,
    dust_likelihood_serial_fallbacks, dust_likelihood_server,
    dust_likelihood_set_rng_state, dust_likelihood_set_step_shape,
    dust_likelihood_step_shape, dust_ode_control,
    dust_system_compare_data, dust_system_create, dust_system_internals,
    dust_system_reorder, dust_system_rng_state, dust_system_run_to_time,
    dust_system_set_rng_state, dust_system_set_state,
    dust_system_set_state_initial, dust_system_set_time,
    dust_system_simulate, dust_system_state, dust_system_time,
    dust_system_update_pars, dust_unfilter_create, dust_unpack_index,
    dust_unpack_state, logistic, malaria,
    resample_weight, rng_streams,
    scale_log_weights, seir_age, sir, sir_cases, sirode, sirs, walk)

__all__ = [
    "DustError", "DustLikelihood", "DustServer", "DustSystem",
    "DustUnfilter", "Generator",
    "device_count", "dust_filter_create", "dust_filter_data",
    "dust_likelihood_last_gradient",
    "dust_likelihood_last_snapshots", "dust_likelihood_last_state",
    "dust_likelihood_last_trajectories",
    "dust_likelihood_rng_state",
    "dust_likelihood_run", "dust_likelihood_serial_fallbacks",
    "dust_likelihood_set_step_shape", "dust_likelihood_step_shape",
    "dust_likelihood_server", "dust_likelihood_set_rng_state",
    "dust_ode_control",
    "dust_system_compare_data", "dust_system_create",
    "dust_system_internals", "dust_system_reorder", "dust_system_rng_state",
    "dust_system_run_to_time", "dust_system_set_rng_state",
    "dust_system_set_state", "dust_system_set_state_initial",
    "dust_system_set_time", "dust_system_simulate", "dust_system_state",
    "dust_system_time", "dust_system_update_pars", "dust_unfilter_create",
    "dust_unpack_index", "dust_unpack_state",
    "logistic", "malaria",
    "resample_weight", "rng_streams", "scale_log_weights", "seir_age", "sir",
    "sir_cases", "sirode", "sirs", "walk"]
