"""GB300 (sm_103a) backend for the CTMRG hot path of Ace-TN.

Import name: ``acetn_gb300`` (``pip install .`` maps the source directory
``ace-tn_gb300`` to it; in-tree, the repository's test and bench entry points
import the directory and register the same alias).

Drop-in replacements for the reference's CTMRG-path objects, operating on
any iPEPS object with the reference's access pattern whose tensors are
float64 CUDA tensors:

    ctmrg(ipeps, config)          acetn/renormalization/ctmrg.py
    DirectionalMover(config)      acetn/renormalization/directional_mover.py
    ProjectorCalculator(config)   acetn/renormalization/projectors.py
    RDM(ipeps), measure(...)      acetn/measurement/
    svd_lowrank, fused_*          acetn/linalg/
    build_norm_tensor, absorb_bond  acetn/evolution/ (full_update.py, fast_full_update.py)
    ALSSolver                     acetn/evolution/als_solver.py

All arithmetic runs in libctm_gb300.so; there is no CPU fallback.
"""

from . import _abi
from ._abi import autotune, autotune_table, set_mixed_contraction
from ._build import build
from .config import CTMRGConfig
from .ctmrg import ctmrg, pair_order, sweep_order
from .directional_mover import DirectionalMover
from .als import ALSSolver
from .batched import BatchedCTMRG
from .full_update import absorb_bond, build_norm_tensor
from .graph import CTMRGGraph
from .linalg import (fused_3matmul_svd_lowrank, fused_matmul_svd_lowrank, matmul, qr, svd,
                     svd_lowrank)
from .measure import measure
from .models import HeisenbergModel, IsingModel
from .projectors import ProjectorCalculator
from .rdm import RDM
from .state import Bond, IpepsState, random_state

__all__ = ["build", "CTMRGConfig", "ctmrg", "sweep_order", "pair_order", "DirectionalMover",
           "ProjectorCalculator", "CTMRGGraph", "BatchedCTMRG", "RDM", "measure", "svd_lowrank", "fused_matmul_svd_lowrank",
           "fused_3matmul_svd_lowrank", "qr", "svd", "matmul", "HeisenbergModel", "IsingModel",
           "Bond", "IpepsState", "random_state", "build_norm_tensor", "absorb_bond",
           "autotune", "autotune_table", "set_mixed_contraction", "ALSSolver"]
