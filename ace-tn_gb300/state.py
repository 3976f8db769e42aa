"""Device-resident iPEPS state with the reference's access pattern.

``IpepsState`` stores, per site, ``{'A': A, 'C': [C0..C3], 'E': [E0..E3]}``
as float64 CUDA tensors and is indexed like ``TensorNetwork``
(acetn/ipeps/tensor_network.py:33-56): ``state[(x, y)]['C'][k]``.  Unlike the
reference's class-level site dictionary (tensor_network.py:12), every
instance owns its tensors.  ``site_list`` / ``bond_list`` follow
tensor_network.py:153-193.
"""

import pickle
import types
from dataclasses import dataclass

import numpy as np
import torch


@dataclass(frozen=True)
class Bond:
    """acetn/ipeps/bond.py:4-22."""
    s1: tuple
    s2: tuple
    k: int

    def __post_init__(self):
        object.__setattr__(self, "s1", tuple(self.s1))
        object.__setattr__(self, "s2", tuple(self.s2))

    def __iter__(self):
        return iter((self.s1, self.s2, self.k))


def build_site_list(nx, ny):
    return [(xi, yi) for xi in range(nx) for yi in range(ny)]


def build_bond_list(nx, ny):
    bonds = []
    for xi in range(nx):
        for yi in range(ny):
            bonds.append(Bond((xi, yi), ((xi + 1) % nx, yi), 2))
    for yi in range(ny):
        for xi in range(nx):
            bonds.append(Bond((xi, yi), (xi, (yi + 1) % ny), 1))
    return bonds


class IpepsState:
    def __init__(self, nx, ny, dims, device="cuda"):
        self.nx, self.ny = nx, ny
        self.dims = dict(dims)
        self.device = torch.device(device)
        self.dtype = torch.float64
        self.site_list = build_site_list(nx, ny)
        self.bond_list = build_bond_list(nx, ny)
        self._sites = {}
        self.rank = 0
        self.is_distributed = False

    def __getitem__(self, site):
        st = self._sites.get(tuple(site))
        if st is None:
            raise ValueError(f"Site tensor not defined at site {site}.")
        return st

    def __setitem__(self, site, value):
        self._sites[tuple(site)] = value

    def set_site(self, site, A, C, E):
        dev = self.device

        def conv(x):
            if isinstance(x, np.ndarray):
                x = torch.from_numpy(np.ascontiguousarray(x))
            return x.to(device=dev, dtype=torch.float64).contiguous().clone()

        self[site] = {"A": conv(A), "C": [conv(c) for c in C], "E": [conv(e) for e in E]}

    @classmethod
    def from_arrays(cls, sites, nx, ny, chi, device="cuda"):
        """``sites``: {(x, y): {'A': array, 'C': [4], 'E': [4]}} (numpy or torch)."""
        first = next(iter(sites.values()))
        D, d = first["A"].shape[0], first["A"].shape[4]
        st = cls(nx, ny, {"phys": d, "bond": D, "chi": chi}, device)
        for s, v in sites.items():
            st.set_site(s, v["A"], v["C"], v["E"])
        return st

    def to_numpy(self):
        return {s: {"A": v["A"].cpu().numpy(), "C": [c.cpu().numpy() for c in v["C"]],
                    "E": [e.cpu().numpy() for e in v["E"]]} for s, v in self._sites.items()}

    def save(self, filename):
        """Plain tensor-dict checkpoint (torch.save of CPU tensors)."""
        data = {"nx": self.nx, "ny": self.ny, "dims": self.dims,
                "sites": {f"{s[0]},{s[1]}": {"A": v["A"].cpu(), "C": [c.cpu() for c in v["C"]],
                                            "E": [e.cpu() for e in v["E"]]}
                          for s, v in self._sites.items()}}
        torch.save(data, filename)

    @classmethod
    def load(cls, filename, device="cuda"):
        data = torch.load(filename, weights_only=True)
        st = cls(data["nx"], data["ny"], data["dims"], device)
        for key, v in data["sites"].items():
            x, y = (int(t) for t in key.split(","))
            st.set_site((x, y), v["A"], v["C"], v["E"])
        return st

    @classmethod
    def load_reference(cls, filename, device="cuda"):
        """Reads a checkpoint written by the reference's ``TensorNetwork.save``
        (acetn/ipeps/tensor_network.py:94-111: torch.save of
        {"tensor_network": ..., "tensors": {site: SiteTensor}}) without
        importing the reference.  The file is unpickled (it holds objects, not
        only tensors), so read only checkpoints from a trusted source."""
        data = torch.load(filename, map_location="cpu", weights_only=False,
                          pickle_module=_REF_PICKLE)
        if not isinstance(data, dict) or "tensors" not in data:
            raise ValueError(f"{filename}: not a checkpoint of the reference's TensorNetwork.save")
        tn, tensors = data.get("tensor_network"), data["tensors"]
        sites = sorted(tuple(s) for s in tensors)
        nx = getattr(tn, "nx", max(s[0] for s in sites) + 1)
        ny = getattr(tn, "ny", max(s[1] for s in sites) + 1)
        A0, C0, _ = _site_arrays(next(iter(tensors.values())))
        dims = dict(getattr(tn, "dims", None) or
                    {"phys": A0.shape[4], "bond": A0.shape[0], "chi": C0[0].shape[0]})
        st = cls(nx, ny, dims, device)
        for site, obj in tensors.items():
            A, C, E = _site_arrays(obj)
            st.set_site(tuple(site), A, C, E)
        return st


class _RefStub:
    """Stand-in for a class of the reference while one of its checkpoints is
    read: pickle rebuilds objects without calling __init__ and restores their
    attributes, which is all a checkpoint needs (SiteTensor._site_tensor,
    _corner_tensors, _edge_tensors; TensorNetwork.nx, ny, dims)."""

    def __new__(cls, *args, **kwargs):
        obj = object.__new__(cls)
        obj._args = args
        return obj

    def __setstate__(self, state):
        if isinstance(state, tuple) and len(state) == 2:  # (dict, slots)
            state = {**(state[0] or {}), **(state[1] or {})}
        if isinstance(state, dict):
            self.__dict__.update(state)
        else:
            self._state = state


class _RefUnpickler(pickle.Unpickler):
    """Unpickler that resolves the reference's classes (module acetn.*) to
    _RefStub subclasses of the same name, so that reading a reference
    checkpoint needs neither the reference nor its dependencies."""

    _stubs = {}

    def find_class(self, module, name):
        if module == "acetn" or module.startswith("acetn."):
            key = (module, name)
            if key not in self._stubs:
                self._stubs[key] = type(name, (_RefStub,), {"__module__": module})
            return self._stubs[key]
        return super().find_class(module, name)


_REF_PICKLE = types.SimpleNamespace(__name__="pickle", Unpickler=_RefUnpickler, load=pickle.load,
                                    Pickler=pickle.Pickler, dump=pickle.dump)


def _site_arrays(obj):
    """(A, [C0..C3], [E0..E3]) of a reference SiteTensor (or its stand-in)."""
    d = obj.__dict__
    if "_site_tensor" in d:
        return d["_site_tensor"], list(d["_corner_tensors"]), list(d["_edge_tensors"])
    return obj["A"], list(obj["C"]), list(obj["E"])


def _initial_environment(a):
    """Initial corner and edge tensors from the site tensor
    (acetn/ipeps/site_tensor.py:152-202)."""
    D = a.shape[0]
    C, E = [], []
    for k in range(4):
        ak = a.permute([(i + k) % 4 for i in range(4)] + [4])
        ck = torch.einsum("lurdp,luRDp->dDrR", ak, ak.conj()).reshape(D * D, D * D)
        C.append((ck / ck.norm()).contiguous())
        ek = torch.einsum("lurdp,LuRDp->lLrRdD", ak, ak.conj()).reshape(D * D, D * D, D, D)
        E.append((ek / ek.norm()).contiguous())
    return C, E


def random_state(D, chi, seed, d=2, nx=2, ny=2, bias=None, device="cuda"):
    """Seeded synthetic iPEPS: per site in ``site_list`` order, A has i.i.d.
    N(0,1) entries from ``numpy.random.default_rng(seed)`` (plus ``bias`` on
    A[0,0,0,0,0] when given), unit Frobenius norm, and the initial
    environment of acetn/ipeps/site_tensor.py:152-202."""
    rng = np.random.default_rng(seed)
    st = IpepsState(nx, ny, {"phys": d, "bond": D, "chi": chi}, device)
    for s in st.site_list:
        a = rng.standard_normal((D, D, D, D, d))
        if bias is not None:
            a[0, 0, 0, 0, 0] += bias
        a = a / np.linalg.norm(a)
        at = torch.from_numpy(a).to(device=st.device)
        C, E = _initial_environment(at)
        st[s] = {"A": at.contiguous(), "C": C, "E": E}
    return st
