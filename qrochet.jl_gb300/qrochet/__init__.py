"""qrochet -- GB300 (sm_103a) implementation of Qrochet.jl's Chain (MPS/MPO) hot path.

Python mirror of the reference's Julia API; every operation runs in libqrochet_gpu.so through
its C ABI (include/qrochet_gpu.h).  ``f!`` in Julia is ``f_`` here.
"""
from ._lib import (ArgumentError, DimensionMismatch, GPUError, MissingSchmidtCoefficientsException,
                   launch_count)
from .chain import (MPO, MPS, pMPS, Chain, Open, Periodic, canonicality_error, canonize, canonize_,
                    canonize_site, canonize_site_, contract_between, contract_between_, device_count,
                    evolve_, evolve_layer_, expect, isleftcanonical, isrightcanonical, mixed_canonize, mixed_canonize_,
                    mpo_expect, norm, normalize_, overlap, truncate, truncate_, zeros_chain, ones_chain, Product,
                    PinnedArray, probe_peak, prof_enable, prof_read, set_device, PROF_KINDS, rand,
                    sampler_bond_dims)
from .dense import Dense, Operator, Scalar, State, gate_from_matrix, validate_gate
from .quantum import inputs, isdual, lanes, ninputs, nlanes, noutputs, nsites, outputs, sites, socket
from .site import Site, nextindex, site
from . import checkpoint

__all__ = [
    "ArgumentError", "DimensionMismatch", "GPUError", "MissingSchmidtCoefficientsException",
    "launch_count", "MPO", "MPS", "pMPS", "Chain", "Open", "Periodic", "canonicality_error", "canonize",
    "canonize_", "canonize_site", "canonize_site_", "contract_between", "contract_between_",
    "device_count", "evolve_", "evolve_layer_", "expect", "isleftcanonical", "isrightcanonical", "mixed_canonize",
    "mixed_canonize_", "mpo_expect", "norm", "normalize_", "overlap", "truncate", "truncate_",
    "zeros_chain", "Dense", "Operator", "State", "gate_from_matrix", "validate_gate", "Site",
    "nextindex", "site", "PinnedArray", "probe_peak", "prof_enable", "prof_read", "set_device",
    "PROF_KINDS", "checkpoint", "rand", "sampler_bond_dims", "Scalar", "inputs", "isdual", "ninputs",
    "noutputs", "nsites", "outputs", "sites", "socket", "lanes", "nlanes", "ones_chain", "Product",
]
