"""CTMRG configuration of the GB300 backend.

Mirrors ``CTMRGConfig`` of the reference (acetn/ipeps/ipeps_config.py:16-24,
documented in docs/source/input_settings.rst:45-54) and adds two fields:

* ``backend``   -- "gb300" selects this library (the reference keeps "torch").
* ``precision`` -- "fp64": every product in FP64, the drop-in path;
                   "mixed": tensor-core range finder and split-precision
                   products feeding the projectors (half- and full-system,
                   rSVD; full-rank: split-precision products, FP64 SVD).
* ``mixed_svd_floor`` -- mixed precision only: singular values below this
                   fraction of the largest are dropped in addition to
                   ``svd_cutoff`` (the reference's 1e-12, which the FP64 path
                   keeps).  Default 1e-6: below about 1e-6 of the largest the
                   spectrum of the 3xBF16 Rayleigh-Ritz product is rounding
                   noise, and keeping it (weighted by s^-1/2) moves converged
                   energies (the Ising ground-state fixture: 4e-5 with a 1e-8
                   floor, within 5e-6 with 1e-6).  Never below 1e-8.
* ``mixed_flags`` -- mixed precision only: CTM_MIXED_* bits of the C ABI
                   selecting higher precision for single stages (3xBF16
                   range finder, FP64 SVD, FP64 quarter tensors, FP32 SIMT
                   products); 0 = the defaults.

Any object with the reference's attribute names works as a config; missing
attributes take the defaults below.
"""

from dataclasses import dataclass
from typing import Literal


@dataclass
class CTMRGConfig:
    steps: int = 40
    projectors: Literal["half-system", "full-system"] = "half-system"
    svd_type: Literal["rsvd", "full-rank"] = "rsvd"
    svd_cutoff: float = 1e-12
    rsvd_niter: int = 2
    rsvd_oversampling: int = 2
    disable_progressbar: bool = False
    backend: Literal["gb300"] = "gb300"
    precision: Literal["fp64", "mixed"] = "fp64"
    mixed_svd_floor: float = 1e-6
    mixed_flags: int = 0


def resolve(config):
    """Returns a ``CTMRGConfig`` from a dict, a reference config object or None."""
    if config is None:
        return CTMRGConfig()
    if isinstance(config, CTMRGConfig):
        return config
    if isinstance(config, dict):
        return CTMRGConfig(**config)
    fields = CTMRGConfig.__dataclass_fields__
    return CTMRGConfig(**{k: getattr(config, k) for k in fields if hasattr(config, k)})
