"""The reference's own objects through the dispatch lines of INTEGRATION.md.

The reference is installed (pure Python, no extension) into baseline/_ref by
``pip install --no-deps --target baseline/_ref <reference>`` (with tqdm beside
it); its ``toml`` import is served by a stand-in on the standard library's
``tomllib``.  The tests skip when that install is absent.

* CPU: with ``backend="gb300"`` the reference's ``ctmrg`` and ``measure``
  (patched exactly as INTEGRATION.md shows) reach this package, which raises
  on CPU tensors: there is no fallback to the torch path.  With ``"torch"``
  the reference's own path runs unchanged.
* GPU: a reference ``Ipeps`` on CUDA, renormalized by this package through
  the dispatch (full-rank SVD, so no random test matrices are involved),
  gives the energy and the bond RDMs of the reference's own torch path on
  the same device to 1e-10.
"""

import importlib
import os
import sys
import tomllib
import types

import numpy as np
import pytest
import torch

import acetn_gb300 as gb

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.path.join(ROOT, "baseline", "_ref")


def _toml_stand_in():
    mod = types.ModuleType("toml")

    def load(f):
        if isinstance(f, str):
            with open(f, "rb") as fh:
                return tomllib.load(fh)
        return tomllib.load(f)

    mod.load = load
    mod.loads = tomllib.loads
    mod.dumps = lambda d: repr(d) + "\n"
    return mod


@pytest.fixture(scope="module")
def acetn():
    if not os.path.isdir(os.path.join(REF, "acetn")):
        pytest.skip("the reference is not installed in baseline/_ref")
    sys.modules.setdefault("toml", _toml_stand_in())
    if REF not in sys.path:
        sys.path.append(REF)
    mods = types.SimpleNamespace(
        ipeps=importlib.import_module("acetn.ipeps.ipeps"),
        ctmrg=importlib.import_module("acetn.renormalization.ctmrg"),
        measure=importlib.import_module("acetn.measurement.measure"),
        models=importlib.import_module("acetn.model.model_factory"))
    yield mods


@pytest.fixture
def dispatched(acetn):
    """Applies the dispatch of INTEGRATION.md section 3 to the reference
    (in its ctmrg.py and measure.py, and where ipeps.py imported them)."""
    torch_ctmrg, torch_measure = acetn.ctmrg.ctmrg, acetn.measure.measure

    def ctmrg(ipeps, config):
        if getattr(config, "backend", "torch") == "gb300":
            return gb.ctmrg(ipeps, config)
        return torch_ctmrg(ipeps, config)

    def measure(ipeps, model):
        if getattr(ipeps.config.ctmrg, "backend", "torch") == "gb300":
            return gb.measure(ipeps, model)
        return torch_measure(ipeps, model)

    acetn.ctmrg.ctmrg = acetn.ipeps.ctmrg = ctmrg
    acetn.measure.measure = acetn.ipeps.measure = measure
    yield acetn
    acetn.ctmrg.ctmrg = acetn.ipeps.ctmrg = torch_ctmrg
    acetn.measure.measure = acetn.ipeps.measure = torch_measure


def make_ipeps(acetn, device, backend, D=2, chi=8, steps=3, seed=5):
    """A reference Ipeps with seeded N(0,1) site tensors (unit norm) and the
    reference's initial boundary tensors built from them."""
    cfg = {"TN": {"nx": 2, "ny": 2, "dims": {"phys": 2, "bond": D, "chi": chi}},
           "dtype": "float64", "device": device,
           "ctmrg": {"steps": steps, "svd_type": "full-rank", "disable_progressbar": True},
           "model": {"name": "heisenberg", "params": {"J": 1.0}}}
    ip = acetn.ipeps.Ipeps(cfg)
    ip.config.ctmrg.backend = backend
    g = torch.Generator().manual_seed(seed)
    for s in ip.site_list:
        a = torch.randn(D, D, D, D, 2, generator=g, dtype=torch.float64)
        ip[s]["A"] = (a / a.norm()).to(device)
        ip[s].initialize_corner_tensors()
        ip[s].initialize_edge_tensors()
    return ip


def test_gb300_backend_reaches_this_package_and_refuses_cpu_tensors(dispatched):
    ip = make_ipeps(dispatched, "cpu", "gb300")
    with pytest.raises(ValueError, match="CUDA tensor"):
        ip.renormalize()
    model = dispatched.models.model_factory.create(ip.config.model)
    with pytest.raises(ValueError, match="CUDA tensor"):
        ip.measure(model)


def test_torch_backend_runs_the_reference_path(dispatched):
    ip = make_ipeps(dispatched, "cpu", "torch", steps=1)
    ip.renormalize()
    model = dispatched.models.model_factory.create(ip.config.model)
    e = float(ip.measure(model)["Energy"])
    assert np.isfinite(e)
    assert tuple(ip[(0, 0)]["C"][0].shape) == (8, 8)  # grown from D^2 = 4 to chi


@pytest.mark.gpu
def test_reference_ipeps_on_gpu_through_the_dispatch_matches_its_torch_path(dispatched):
    gb.build()
    results = {}
    # the reference's site dictionary is shared by all Ipeps objects, so the
    # two runs use it one after the other
    for backend in ("torch", "gb300"):
        ip = make_ipeps(dispatched, "cuda", backend, D=3, chi=12, steps=6)
        ip.renormalize()
        model = dispatched.models.model_factory.create(ip.config.model)
        e = float(ip.measure(model)["Energy"])
        rdm = gb.RDM(ip)
        bonds = []
        for b in ip.bond_list:
            r = rdm[b].cpu().numpy()
            bonds.append(r / np.einsum("pqpq->", r))
        results[backend] = (e, bonds, ip[(0, 0)]["C"][0].dtype, ip[(0, 0)]["C"][0].device)
    e_t, b_t, _, _ = results["torch"]
    e_g, b_g, dt, dev = results["gb300"]
    assert dt == torch.float64 and dev.type == "cuda"
    assert abs(e_g - e_t) <= 1e-10 * abs(e_t)
    for x, y in zip(b_g, b_t):
        assert np.abs(x - y).max() < 1e-10
    assert gb._abi.device_status() == 0
