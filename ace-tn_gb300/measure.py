"""Measurement on the GB300 library.

Mirror of ``measure(ipeps, model)`` (acetn/measurement/measure.py:5-198):
energy per site and averaged observables from trace-normalised RDMs.  The
RDMs are built on the GPU; the d x d (d^4) contractions with the operators
are tiny and done with torch on the same device.  ``verbose`` prints the
reference's tables with tqdm.write.
"""

import torch
from ._progress import tqdm

from .rdm import RDM


def _mat(op):
    return op.mat if hasattr(op, "mat") else op


def measure(ipeps, model, verbose=True, precision="fp64"):
    """``precision="mixed"`` builds the RDMs on tensor cores (bond) and in
    FP32 (site); the normalisations and operator contractions stay FP64."""
    out = {"Energy": 0.0}
    rdm = RDM(ipeps, precision)
    site_list, bond_list = ipeps.site_list, ipeps.bond_list
    dim = model.dim
    one_keys = list(model.one_site_observables((0, 0)).keys())
    for key in one_keys:
        out[key] = 0.0
    for site in site_list:
        r = rdm[site]
        norm = torch.einsum("pp->", r).real
        h1 = model.one_site_hamiltonian(site)
        if h1 is not None:
            h1 = _mat(h1).to(device=r.device, dtype=r.dtype)
            out["Energy"] += torch.einsum("Pp,pP->", r, h1).real / norm
        line = f"{site}"
        for name, op in model.one_site_observables(site).items():
            v = torch.einsum("Pp,pP->", r, _mat(op).to(device=r.device, dtype=r.dtype)).real / norm
            out[name] += v
            line += f"\t{v.item():.8f}"
        if verbose and one_keys:
            tqdm.write(line)
    for key in one_keys:
        out[key] /= len(site_list)
    two_keys = list(model.two_site_observables(bond_list[0]).keys())
    for key in two_keys:
        out[key] = 0.0
    for bond in bond_list:
        r = rdm[bond]
        norm = torch.einsum("pqpq->", r).real
        h2 = _mat(model.two_site_hamiltonian(bond)).reshape((dim,) * 4).to(device=r.device,
                                                                           dtype=r.dtype)
        out["Energy"] += torch.einsum("PQpq,pqPQ->", r, h2).real / norm
        for name, op in model.two_site_observables(bond).items():
            op = _mat(op).reshape((dim,) * 4).to(device=r.device, dtype=r.dtype)
            out[name] += torch.einsum("PQpq,pqPQ->", r, op).real / norm
    for key in two_keys:
        out[key] /= len(bond_list)
    out["Energy"] /= len(site_list)
    if verbose:
        tqdm.write("Measurement averages:")
        tqdm.write("\n".join(f"{key}: {value}" for key, value in out.items()))
    return out
