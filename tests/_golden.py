"""Loading of the golden vectors in tests/golden (written by make_golden.py)."""

import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SITES = [(0, 0), (0, 1), (1, 0), (1, 1)]


def load(name):
    return np.load(os.path.join(GOLDEN, name))


def site_arrays(z, prefix="in"):
    out = {}
    for s in SITES:
        t = f"{prefix}_{s[0]}{s[1]}"
        out[s] = {"A": z[t + "_A"], "C": [z[f"{t}_C{k}"] for k in range(4)],
                  "E": [z[f"{t}_E{k}"] for k in range(4)]}
    return out


def oracle_state(z, chi, prefix="in"):
    from oracle import ctm_oracle as orc
    return orc.OracleState(site_arrays(z, prefix), 2, 2, chi)


def gpu_state(z, chi, prefix="in"):
    import acetn_gb300 as gb
    return gb.IpepsState.from_arrays(site_arrays(z, prefix), 2, 2, chi, device="cuda")


def rel(a, b):
    a = np.asarray(a, dtype=float)
    b = np.asarray(b, dtype=float)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


SITES_K = {0: [(0, 0), (1, 0), (1, 1), (0, 1)], 1: [(0, 0), (0, 1), (1, 1), (1, 0)],
           2: [(0, 0), (1, 0), (1, 1), (0, 1)], 3: [(0, 0), (0, 1), (1, 1), (1, 0)]}


def bond_energies(st):
    """Per-bond Heisenberg <h_b> from trace-normalised FP64 bond RDMs
    (precision bars are set against the largest |<h_b>|)."""
    import torch

    import acetn_gb300 as gb

    rdm = gb.RDM(st)
    model = gb.HeisenbergModel(1.0)
    out = []
    for bd in st.bond_list:
        r = rdm[bd]
        h2 = torch.as_tensor(model.two_site_hamiltonian(bd)).reshape(2, 2, 2, 2).to(r)
        out.append(float(torch.einsum("PQpq,pqPQ->", r, h2) / torch.einsum("pqpq->", r)))
    return np.array(out)
