"""Generate ``norm_tensor_d2.npz``: the full update's norm tensor computed by
the Ace-TN reference itself (``build_norm_tensor`` and
``build_norm_tensor_core_blocked``, acetn/evolution/full_update.py:163-268)
for both bond directions of a seeded 2x2 state, with its inputs, to pin the
oracle's ``norm_tensor``.

Run in a container where the reference source tree is available:

    python tests/golden/make_norm_tensor.py /path/to/ace-tn
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
    from acetn.ipeps import Ipeps
    from acetn.evolution.full_update import build_norm_tensor, build_norm_tensor_core_blocked
    torch.manual_seed(11)
    cfg = {"dtype": "float64", "device": "cpu",
           "TN": {"nx": 2, "ny": 2, "dims": {"phys": 2, "bond": 2, "chi": 6}},
           "model": {"name": "heisenberg", "params": {"J": 1.0}},
           "ctmrg": {"disable_progressbar": True}}
    ip = Ipeps(cfg)
    rng = np.random.default_rng(5)
    D, nD = 2, 4
    out = {}
    for s in ip.site_list:
        key = f"{s[0]}_{s[1]}"
        out[f"{key}_A"] = ip[s]["A"].numpy()
        for k in range(4):
            out[f"{key}_C{k}"] = ip[s]["C"][k].numpy()
            out[f"{key}_E{k}"] = ip[s]["E"][k].numpy()
    for k, (s1, s2) in ((2, ((0, 0), (1, 0))), (1, ((0, 0), (0, 1)))):
        a1q = rng.standard_normal((D, D, D, nD))
        a2q = rng.standard_normal((D, D, D, nD))
        n12 = build_norm_tensor(ip, (s1, s2, k), torch.from_numpy(a1q), torch.from_numpy(a2q))
        t1, t2 = ip[s1], ip[s2]
        nb = build_norm_tensor_core_blocked(
            t1["C"][(k + 1) % 4], t1["E"][(k + 1) % 4], t1["E"][k % 4], t1["C"][(k + 2) % 4],
            t1["E"][(k + 2) % 4], torch.from_numpy(a1q),
            t2["C"][k % 4], t2["E"][k % 4], t2["E"][(k + 3) % 4], t2["C"][(k + 3) % 4],
            t2["E"][(k + 2) % 4], torch.from_numpy(a2q))
        out[f"k{k}_a1q"], out[f"k{k}_a2q"] = a1q, a2q
        out[f"k{k}_n12"], out[f"k{k}_n12_blocked"] = n12.numpy(), nb.numpy()
    np.savez(os.path.join(HERE, "norm_tensor_d2.npz"), **out)
    print("wrote norm_tensor_d2.npz", out["k2_n12"].shape)


if __name__ == "__main__":
    main(sys.argv[1])
