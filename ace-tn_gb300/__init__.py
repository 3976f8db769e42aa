"""GB300 (sm_103a) backend for the CTMRG hot path of Ace-TN.

Import name: the directory is ``ace-tn_gb300``; import it with
``importlib.import_module("ace-tn_gb300")`` (the repository's test and bench
entry points also register the alias ``acetn_gb300``).

Drop-in replacements for the reference's CTMRG-path objects, operating on
any iPEPS object with the reference's access pattern whose tensors are
float64 CUDA tensors:

    ctmrg(ipeps, config)          acetn/renormalization/ctmrg.py
    DirectionalMover(config)      acetn/renormalization/directional_mover.py
    ProjectorCalculator(config)   acetn/renormalization/projectors.py
    RDM(ipeps), measure(...)      acetn/measurement/
    svd_lowrank, fused_*          acetn/linalg/

All arithmetic runs in libctm_gb300.so; there is no CPU fallback.
"""

from . import _abi
from ._build import build
from .config import CTMRGConfig
from .ctmrg import ctmrg, sweep_order
from .directional_mover import DirectionalMover
from .graph import CTMRGGraph
from .linalg import (fused_3matmul_svd_lowrank, fused_matmul_svd_lowrank, matmul, qr, svd,
                     svd_lowrank)
from .measure import measure
from .models import HeisenbergModel, IsingModel
from .projectors import ProjectorCalculator
from .rdm import RDM
from .state import Bond, IpepsState, random_state

__all__ = ["build", "CTMRGConfig", "ctmrg", "sweep_order", "DirectionalMover",
           "ProjectorCalculator", "CTMRGGraph", "RDM", "measure", "svd_lowrank", "fused_matmul_svd_lowrank",
           "fused_3matmul_svd_lowrank", "qr", "svd", "matmul", "HeisenbergModel", "IsingModel",
           "Bond", "IpepsState", "random_state"]
