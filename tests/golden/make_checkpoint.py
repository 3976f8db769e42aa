"""Generate ``ref_checkpoint_d2.pt`` (a checkpoint written by the Ace-TN
reference's own ``TensorNetwork.save``, acetn/ipeps/tensor_network.py:94-111)
and ``ref_checkpoint_d2.npz`` (the same tensors as plain arrays), the
fixtures of the checkpoint-interop tests.

Run in a container where the reference source tree is available:

    python tests/golden/make_checkpoint.py /path/to/ace-tn

The state: a 2x2 Heisenberg iPEPS with D=2, chi=6 as the reference
initialises it (seeded site tensors; C and E from them, D^2 = 4 wide).
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import _install_toml_stub  # noqa: E402


def main(ref_root):
    _install_toml_stub()
    sys.path.insert(0, ref_root)
    import torch
    torch.manual_seed(7)
    from acetn.ipeps import Ipeps
    cfg = {"dtype": "float64", "device": "cpu",
           "TN": {"nx": 2, "ny": 2, "dims": {"phys": 2, "bond": 2, "chi": 6}},
           "model": {"name": "heisenberg", "params": {"J": 1.0}},
           "ctmrg": {"disable_progressbar": True}}
    ip = Ipeps(cfg)
    pt = os.path.join(HERE, "ref_checkpoint_d2.pt")
    ip.save(pt)
    arrays = {}
    for s in ip.site_list:
        key = f"{s[0]}_{s[1]}"
        arrays[f"{key}_A"] = ip[s]["A"].numpy()
        for k in range(4):
            arrays[f"{key}_C{k}"] = ip[s]["C"][k].numpy()
            arrays[f"{key}_E{k}"] = ip[s]["E"][k].numpy()
    np.savez(os.path.join(HERE, "ref_checkpoint_d2.npz"), **arrays)
    print("wrote", pt, {k: v.shape for k, v in list(arrays.items())[:3]})


if __name__ == "__main__":
    main(sys.argv[1])
