"""The two built-in models of the reference as operator tables.

Same Hamiltonians and observables as ``IsingModel`` and ``HeisenbergModel``
(acetn/model/models/ising.py:4-21, heisenberg.py:4-26) with the real Pauli-Y
convention of acetn/model/pauli_matrix.py (a product of two real Y matrices
carries phase -1), exposing the methods ``measure`` calls.  Reference model
objects can be passed to ``measure`` unchanged.
"""

import torch

_X = [[0.0, 1.0], [1.0, 0.0]]
_Yr = [[0.0, -1.0], [1.0, 0.0]]
_Z = [[1.0, 0.0], [0.0, -1.0]]


def _t(m, device):
    return torch.tensor(m, dtype=torch.float64, device=device)


class _Model:
    dim = 2

    def __init__(self, device="cpu", **params):
        self.device = torch.device(device)
        self.params = params

    def one_site_observables(self, site):
        return {}

    def two_site_observables(self, bond):
        return {}

    def one_site_hamiltonian(self, site):
        return None


class HeisenbergModel(_Model):
    def __init__(self, J=1.0, device="cpu"):
        super().__init__(device, J=J)

    def one_site_observables(self, site):
        sgn = 1.0 if (site[0] + site[1]) % 2 == 0 else -1.0
        return {"sx": sgn * _t(_X, self.device), "sz": sgn * _t(_Z, self.device)}

    def two_site_hamiltonian(self, bond):
        X, Y, Z = _t(_X, self.device), _t(_Yr, self.device), _t(_Z, self.device)
        return 0.25 * self.params["J"] * (torch.kron(X, X) - torch.kron(Y, Y) + torch.kron(Z, Z))


class IsingModel(_Model):
    def __init__(self, jz=1.0, hx=3.0, device="cpu"):
        super().__init__(device, jz=jz, hx=hx)

    def one_site_observables(self, site):
        return {"sx": _t(_X, self.device), "sz": _t(_Z, self.device)}

    def one_site_hamiltonian(self, site):
        return -self.params["hx"] * _t(_X, self.device)

    def two_site_hamiltonian(self, bond):
        Z = _t(_Z, self.device)
        return -self.params["jz"] * torch.kron(Z, Z)
