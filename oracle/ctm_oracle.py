"""CPU restatement (numpy, float64) of Ace-TN's CTMRG hot path.

TEST INFRASTRUCTURE ONLY.  This module is the parity oracle: it is imported by
``tests/``, by ``__graft_entry__.smoke()`` and by the ``cpu_baseline`` /
``--impl reference`` legs of ``bench.py``, and nowhere else.  The product path
(the ``ace-tn_gb300`` package and its CUDA library) never imports it and never
falls back to it.

Parity is pinned: ``tests/golden/make_golden.py`` runs the reference itself
(imported read-only in the build container) on seeded inputs with a shared
random-matrix stream and stores its outputs in ``tests/golden/*.npz``; the CPU
test-suite checks this module against those vectors and against the
reference's converged ground-state energies (``tests/integration/ipeps_gs/
energies.csv`` of the reference).

Every function below cites the reference file:line whose algorithm it restates
(paths relative to the reference project root).  The random matrices Omega that
the reference draws inside its randomized SVD (``torch.randn``) are supplied
here by an explicit ``omega(n, q)`` callable, so that the oracle, the reference
and the GPU path can be fed the same matrices.
"""

import contextlib

import numpy as np

try:  # small LAPACK calls are far slower with many BLAS threads
    from threadpoolctl import threadpool_limits as _threadpool_limits
except ImportError:  # pragma: no cover - not installed everywhere
    _threadpool_limits = None

__all__ = [
    "OmegaStream", "bond_permute", "initial_corner_tensors", "initial_edge_tensors",
    "make_quarter_tensor", "svd_lowrank", "fused_matmul_svd_lowrank",
    "fused_3matmul_svd_lowrank", "calculate_projectors", "calculate_half_system",
    "calculate_full_system", "renormalize_cj1", "renormalize_cj2", "renormalize_ej",
    "OracleState", "Mover", "ctmrg", "site_rdm", "bond_rdm", "heisenberg_model",
    "ising_model", "measure", "build_bond_list", "build_site_list", "random_state",
    "norm_tensor", "als_initialize", "als_cost", "als_solve",
]


def _ein(spec, *ops):
    return np.einsum(spec, *ops, optimize=True)


class OmegaStream:
    """Deterministic stream of N(0,1) matrices: call ``i`` draws from
    ``numpy.random.default_rng((seed, i))``.  Stands in for the ``torch.randn``
    draws at ``acetn/linalg/fused_matmul_svd_lowrank.py:32``,
    ``acetn/linalg/fused_3matmul_svd_lowrank.py:34`` and
    ``acetn/linalg/svd_lowrank.py:32``."""

    def __init__(self, seed):
        self.seed = int(seed)
        self.count = 0

    def __call__(self, n, q):
        rng = np.random.default_rng((self.seed, self.count))
        self.count += 1
        return rng.standard_normal((n, q))


# ---------------------------------------------------------------- site tensors

def bond_permute(a, k):
    """``SiteTensor.bond_permute`` (acetn/ipeps/site_tensor.py:138-150)."""
    return np.transpose(a, [(i + k) % 4 for i in range(4)] + [4])


def initial_corner_tensors(a):
    """``SiteTensor.initialize_corner_tensors`` (acetn/ipeps/site_tensor.py:152-174)."""
    bD = a.shape[0]
    out = []
    for k in range(4):
        ak = bond_permute(a, k)
        ck = _ein("lurdp,luRDp->dDrR", ak, np.conj(ak)).reshape(bD**2, bD**2)
        out.append(ck / np.linalg.norm(ck))
    return out


def initial_edge_tensors(a):
    """``SiteTensor.initialize_edge_tensors`` (acetn/ipeps/site_tensor.py:176-202)."""
    bD = a.shape[0]
    out = []
    for k in range(4):
        ak = bond_permute(a, k)
        ek = _ein("lurdp,LuRDp->lLrRdD", ak, np.conj(ak)).reshape(bD**2, bD**2, bD, bD)
        out.append(ek / np.linalg.norm(ek))
    return out


# ---------------------------------------------------------------- projectors

def make_quarter_tensor(site, k):
    """Enlarged corner ``ProjectorCalculator.make_quarter_tensor``
    (acetn/renormalization/projectors.py:35-60).  Returns the (chi*D*D, chi*D*D)
    matrix normalised by its largest |entry| and the 6-leg shape."""
    ak = bond_permute(site["A"], k)
    ck = site["C"][k % 4]
    ek1 = site["E"][(3 + k) % 4]
    ek2 = site["E"][k % 4]
    qk = _ein("ab,bcuU->acuU", ck, ek2)
    qk = _ein("acuU,ealL->cuUelL", qk, ek1)
    qk = _ein("cuUelL,LURDP->cuelRDP", qk, np.conj(ak))
    qk = _ein("lurdp,cuelRDp->crRedD", ak, qk)
    qD = qk.shape
    qk = qk.reshape(qD[0] * qD[1] * qD[2], qD[3] * qD[4] * qD[5])
    qk = qk / np.abs(qk).max()
    return qk, qD


def _few_threads(*arrays):
    if _threadpool_limits is not None and max(a.size for a in arrays) < 1 << 20:
        return _threadpool_limits(limits=1)
    return contextlib.nullcontext()


def _svd(a, full_matrices):
    with _few_threads(a):
        return np.linalg.svd(a, full_matrices=full_matrices)


def _qr_q(y):
    with _few_threads(y):
        return np.linalg.qr(y, mode="reduced")[0]


def svd_lowrank(a, q, niter, omega):
    """``svd_lowrank`` (acetn/linalg/svd_lowrank.py:4-44)."""
    m, n = a.shape
    q = min(q, m, n)
    y = a @ omega(n, q)
    for _ in range(niter):
        y = _qr_q(y)
        y = a @ (a.conj().T @ y)
    qm = _qr_q(y)
    b = qm.conj().T @ a
    ub, s, vh = _svd(b, False)
    return qm @ ub, s, vh.conj().T


def fused_matmul_svd_lowrank(a, b, q, niter, omega):
    """Randomized SVD of ``a @ b`` without forming the product,
    ``fused_matmul_svd_lowrank`` (acetn/linalg/fused_matmul_svd_lowrank.py:4-52)."""
    m = a.shape[0]
    n = b.shape[1]
    q = min(q, m, n)
    y = a @ (b @ omega(n, q))
    for _ in range(niter):
        y = _qr_q(y)
        y = a @ (b @ (b.conj().T @ (a.conj().T @ y)))
    qm = _qr_q(y)
    bp = (qm.conj().T @ a) @ b
    ub, s, vh = _svd(bp, False)
    return qm @ ub, s, vh.conj().T


def fused_3matmul_svd_lowrank(a, b, c, d, q, niter, omega):
    """Randomized SVD of ``a @ b @ c @ d``,
    ``fused_3matmul_svd_lowrank`` (acetn/linalg/fused_3matmul_svd_lowrank.py:4-56)."""
    m = a.shape[0]
    n = d.shape[1]
    q = min(q, m, n)
    y = a @ (b @ (c @ (d @ omega(n, q))))
    for _ in range(niter):
        y = _qr_q(y)
        y = d.conj().T @ (c.conj().T @ (b.conj().T @ (a.conj().T @ y)))
        y = _qr_q(y)
        y = a @ (b @ (c @ (d @ y)))
    qm = _qr_q(y)
    bp = (((qm.conj().T @ a) @ b) @ c) @ d
    ub, s, vh = _svd(bp, False)
    return qm @ ub, s, vh.conj().T


def _truncate(u, s, v, chi, cutoff):
    """Shared truncation of ``calculate_projectors`` / ``calculate_half_system``
    (acetn/renormalization/projectors.py:129-132, 163-167, 203-207)."""
    s = s / s[0]
    c = int(min(chi, int((s > cutoff).sum())))
    u = u[:, :c] * (1.0 / np.sqrt(s[:c]))
    v = v[:, :c] * (1.0 / np.sqrt(s[:c]))
    return u, v, c


def calculate_projectors(r1, r2, f, chi, cfg, omega):
    """``ProjectorCalculator.calculate_projectors`` + ``svd``
    (acetn/renormalization/projectors.py:114-136, 219-236)."""
    if cfg["svd_type"] == "full-rank":
        u, s, vh = _svd(f, True)
        v = vh.conj().T
    else:
        u, s, v = svd_lowrank(f, chi + cfg["rsvd_oversampling"], cfg["rsvd_niter"], omega)
    u, v, c = _truncate(u, s, v, chi, cfg["svd_cutoff"])
    proj1 = _ein("xedD,xz->edDz", r1, np.conj(u))
    proj2 = _ein("cuUy,yz->cuUz", r2, v)
    return proj1, proj2


def calculate_half_system(st, sites, k, cfg, omega):
    """``ProjectorCalculator.calculate_half_system``
    (acetn/renormalization/projectors.py:138-174; full-rank branch via
    ``contract_half_system`` :62-82)."""
    chi = st.chi
    s1, s4 = sites[0], sites[3]
    q1, q1D = make_quarter_tensor(st[s1], k)
    q4, q4D = make_quarter_tensor(st[s4], k + 3)
    if cfg["svd_type"] == "full-rank":
        r = q1 @ q4
        r = r / np.abs(r).max()
        return calculate_projectors(q1.reshape(q1.shape[0], *q1D[3:]),
                                    q4.reshape(*q4D[:3], q4.shape[1]), r, chi, cfg, omega)
    q = chi + cfg["rsvd_oversampling"]
    u, s, v = fused_matmul_svd_lowrank(q1, q4, q, cfg["rsvd_niter"], omega)
    u, v, c = _truncate(u, s, v, chi, cfg["svd_cutoff"])
    q1 = q1.reshape(q1.shape[0], *q1D[3:])
    q4 = q4.reshape(*q4D[:3], q4.shape[1])
    proj1 = _ein("xedD,xz->edDz", q1, np.conj(u))
    proj2 = _ein("cuUy,yz->cuUz", q4, v)
    return proj1, proj2


def calculate_full_system(st, sites, k, cfg, omega):
    """``ProjectorCalculator.calculate_full_system``
    (acetn/renormalization/projectors.py:176-217; full-rank branch via
    ``contract_full_system`` :84-112)."""
    chi = st.chi
    s1, s2, s3, s4 = sites
    q1, q1D = make_quarter_tensor(st[s1], k)
    q2, _ = make_quarter_tensor(st[s2], k + 1)
    q3, _ = make_quarter_tensor(st[s3], k + 2)
    q4, q4D = make_quarter_tensor(st[s4], k + 3)
    if cfg["svd_type"] == "full-rank":
        r1 = q2 @ q1
        r2 = q4 @ q3
        r1 = r1 / np.abs(r1).max()
        r2 = r2 / np.abs(r2).max()
        f = r1 @ r2
        f = f / np.abs(f).max()
        return calculate_projectors(r1.reshape(r1.shape[0], *q1D[3:]),
                                    r2.reshape(*q4D[:3], r2.shape[1]), f, chi, cfg, omega)
    q = chi + cfg["rsvd_oversampling"]
    u, s, v = fused_3matmul_svd_lowrank(q2, q1, q4, q3, q, cfg["rsvd_niter"], omega)
    u, v, c = _truncate(u, s, v, chi, cfg["svd_cutoff"])
    proj1 = (q1.conj().T @ (q2.conj().T @ np.conj(u))).reshape(*q1D[3:], c)
    proj2 = (q4 @ (q3 @ v)).reshape(*q4D[:3], c)
    return proj1, proj2


# ---------------------------------------------------------------- renormalization

def renormalize_cj1(ci, ei, proj):
    """``DirectionalMover.renormalize_cj1`` (acetn/renormalization/directional_mover.py:305-323)."""
    cj = _ein("ablL,bc->alLc", ei, ci)
    cj = _ein("alLc,clLx->ax", cj, proj)
    return cj / np.linalg.norm(cj)


def renormalize_cj2(ci, ei, proj):
    """``DirectionalMover.renormalize_cj2`` (acetn/renormalization/directional_mover.py:325-343)."""
    cj = _ein("ab,bcrR->acrR", ci, ei)
    cj = _ein("arRx,acrR->xc", proj, cj)
    return cj / np.linalg.norm(cj)


def renormalize_ej(ei, ai, proj2, proj1):
    """``DirectionalMover.renormalize_ej`` (acetn/renormalization/directional_mover.py:345-366)."""
    ej = _ein("ablL,buUx->alLuUx", ei, proj1)
    ej = _ein("LURDP,alLuUx->RDPalux", np.conj(ai), ej)
    ej = _ein("lurdp,RDpalux->rdRDax", ai, ej)
    ej = _ein("rdRDax,adDy->yxrR", ej, proj2)
    return ej / np.linalg.norm(ej)


class OracleState:
    """Site-tensor container with the access pattern of the reference's
    ``TensorNetwork`` / ``SiteTensor`` (acetn/ipeps/tensor_network.py:33-56,
    acetn/ipeps/site_tensor.py:41-83): ``st[(x, y)]['A' | 'C' | 'E']``."""

    def __init__(self, sites, nx, ny, chi):
        self.sites = sites
        self.nx, self.ny, self.chi = nx, ny, chi

    def __getitem__(self, s):
        if s not in self.sites:
            raise ValueError(f"Site tensor not defined at site {s}.")
        return self.sites[s]

    def copy(self):
        return OracleState({s: {"A": v["A"].copy(), "C": [c.copy() for c in v["C"]],
                                "E": [e.copy() for e in v["E"]]} for s, v in self.sites.items()},
                           self.nx, self.ny, self.chi)


def random_state(D, chi, seed, d=2, nx=2, ny=2, bias=None):
    """Seeded synthetic site tensors: i.i.d. N(0,1) entries drawn in site order
    ``build_site_list`` (acetn/ipeps/tensor_network.py:179-193), normalised to unit
    Frobenius norm, corner/edge tensors initialised from A as in
    acetn/ipeps/site_tensor.py:152-202.  ``bias`` (optional) is added to the
    up-spin entry A[0,0,0,0,0] before normalising."""
    rng = np.random.default_rng(seed)
    sites = {}
    for s in build_site_list(nx, ny):
        a = rng.standard_normal((D, D, D, D, d))
        if bias is not None:
            a[0, 0, 0, 0, 0] += bias
        a = a / np.linalg.norm(a)
        sites[s] = {"A": a, "C": initial_corner_tensors(a), "E": initial_edge_tensors(a)}
    return OracleState(sites, nx, ny, chi)


class Mover:
    """``DirectionalMover`` (acetn/renormalization/directional_mover.py:5-366),
    non-distributed moves."""

    def __init__(self, cfg, omega):
        self.cfg = cfg
        self.omega = omega
        proj = cfg.get("projectors", "half-system")
        if proj is None or proj == "full-system":
            self.calc = calculate_full_system
        elif proj == "half-system":
            self.calc = calculate_half_system
        else:
            raise ValueError(f"Invalid ctmrg projector type: {proj} provided.")

    def projectors(self, st, sites, k):
        return self.calc(st, sites, k, self.cfg, self.omega)

    @staticmethod
    def move_sites(st, k, idx, n):
        """Site quadruples of ``calculate_{left,up,right,down}_projectors``
        (directional_mover.py:99-181) for row/column ``n`` of move ``k``."""
        nx, ny = st.nx, st.ny
        if k == 0:
            xi, yi = idx, n
            xj, yj = (xi + 1) % nx, (yi - 1 + ny) % ny
            return [(xi, yi), (xj, yi), (xj, yj), (xi, yj)]
        if k == 1:
            xi, yi = n, idx
            xj, yj = (xi - 1 + nx) % nx, (yi - 1 + ny) % ny
            return [(xi, yi), (xi, yj), (xj, yj), (xj, yi)]
        if k == 2:
            xi, yi = idx, n
            xj, yj = (xi - 1 + nx) % nx, (yi + 1) % ny
            return [(xi, yi), (xj, yi), (xj, yj), (xi, yj)]
        xi, yi = n, idx
        xj, yj = (xi + 1) % nx, (yi + 1) % ny
        return [(xi, yi), (xi, yj), (xj, yj), (xj, yi)]

    @staticmethod
    def renorm_targets(st, k, idx, n):
        """(s1, s2, i, j) of the renormalization loops of ``left/up/right/down_move``
        (directional_mover.py:23-97)."""
        nx, ny = st.nx, st.ny
        if k == 0:
            xi, yi = idx, n
            return (xi, yi), ((xi + 1) % nx, yi), yi, (yi + 1) % ny
        if k == 1:
            xi, yi = n, idx
            return (xi, yi), (xi, (yi - 1 + ny) % ny), xi, (xi + 1) % nx
        if k == 2:
            xi, yi = idx, n
            return (xi, yi), ((xi - 1 + nx) % nx, yi), yi, (yi - 1 + ny) % ny
        xi, yi = n, idx
        return (xi, yi), (xi, (yi + 1) % ny), xi, (xi - 1 + nx) % nx

    @staticmethod
    def renormalize_boundary(st, proj1, proj2, s1, s2, i, j, k):
        """``renormalize_boundary`` (directional_mover.py:273-303)."""
        ci = st[s1]["C"][(3 + k) % 4]
        ei = st[s1]["E"][(2 + k) % 4]
        st[s2]["C"][(3 + k) % 4] = renormalize_cj1(ci, ei, proj1[i])
        ci = st[s1]["C"][k]
        ei = st[s1]["E"][k]
        st[s2]["C"][k] = renormalize_cj2(ci, ei, proj2[j])
        ai = bond_permute(st[s1]["A"], k)
        ei = st[s1]["E"][(3 + k) % 4]
        st[s2]["E"][(3 + k) % 4] = renormalize_ej(ei, ai, proj2[i], proj1[j])

    def move(self, st, k, idx):
        """One directional move: all projectors first (phase A), then all
        boundary renormalizations (phase B)."""
        count = st.ny if k in (0, 2) else st.nx
        proj1, proj2 = {}, {}
        for n in range(count):
            proj1[n], proj2[n] = self.projectors(st, self.move_sites(st, k, idx, n), k)
        for n in range(count):
            s1, s2, i, j = self.renorm_targets(st, k, idx, n)
            self.renormalize_boundary(st, proj1, proj2, s1, s2, i, j, k)
        return proj1, proj2

    def left_move(self, st, xi):
        return self.move(st, 0, xi)

    def up_move(self, st, yi):
        return self.move(st, 1, yi)

    def right_move(self, st, xi):
        return self.move(st, 2, xi)

    def down_move(self, st, yi):
        return self.move(st, 3, yi)


def sweep_order(nx, ny):
    """Move order of one CTMRG iteration (acetn/renormalization/ctmrg.py:25-31)."""
    order = []
    for xi in range(nx):
        order.append((0, xi))
        order.append((2, (nx - xi + 1) % nx))
    for yi in range(ny):
        order.append((1, (ny - yi + 1) % ny))
        order.append((3, yi))
    return order


def ctmrg(st, cfg, omega, steps=None):
    """``ctmrg`` (acetn/renormalization/ctmrg.py:4-31), non-distributed branch."""
    mover = Mover(cfg, omega)
    steps = cfg["steps"] if steps is None else steps
    for _ in range(steps):
        for k, idx in sweep_order(st.nx, st.ny):
            mover.move(st, k, idx)
    return st


# ---------------------------------------------------------------- measurement

def site_rdm(site):
    """``RDM.build_site_rdm`` (acetn/measurement/rdm.py:35-67)."""
    c1, c2, c3, c4 = site["C"]
    e1, e2, e3, e4 = site["E"]
    a1 = site["A"]
    tmp1 = _ein("ab,bclL->aclL", c4, e4)
    tmp1 = _ein("aclL,eadD->clLedD", tmp1, e3)
    tmp1 = _ein("clLedD,LURDP->cledURP", tmp1, np.conj(a1))
    tmp2 = _ein("ab,bcuU->acuU", c1, e1)
    tmp3 = _ein("ab,carR->bcrR", c3, e2)
    tmp3 = _ein("ec,bcrR->ebrR", c2, tmp3)
    tmp3 = _ein("ebrR,aeuU->brRauU", tmp3, tmp2)
    tmp3 = _ein("erRcuU,cledURP->ruldP", tmp3, tmp1)
    return _ein("ruldP,lurdp->Pp", tmp3, a1)


def bond_rdm(st, s1, s2, k):
    """``RDM.build_bond_rdm`` + ``build_bond_rdm_core_blocked``
    (acetn/measurement/rdm.py:69-99, 123-153).  The blocked loop of the
    reference only splits the bra physical indices into 1x1 blocks; the
    contraction here is the unblocked form of the same sum
    (``build_bond_rdm_core``, rdm.py:102-120)."""
    t1, t2 = st[s1], st[s2]
    c12 = t1["C"][(k + 1) % 4]; e12 = t1["E"][(k + 1) % 4]; e11 = t1["E"][k % 4]
    c13 = t1["C"][(k + 2) % 4]; e13 = t1["E"][(k + 2) % 4]; a1 = bond_permute(t1["A"], k)
    c21 = t2["C"][k % 4]; e21 = t2["E"][k % 4]; e24 = t2["E"][(k + 3) % 4]
    c24 = t2["C"][(k + 3) % 4]; e23 = t2["E"][(k + 2) % 4]; a2 = bond_permute(t2["A"], k)
    tmp = _ein("ab,bcrR->acrR", c12, e12)
    tmp = _ein("acrR,eauU->crReuU", tmp, e11)
    tmp = _ein("crReuU,LURDP->creuLDP", tmp, np.conj(a1))
    tmp = _ein("creuLDP,lurdp->ceLDPldp", tmp, a1)
    r1 = _ein("ab,bfdD->afdD", c13, e13)
    r1 = _ein("afdD,acLDPldp->fcLPlp", r1, tmp)
    tmp = _ein("ab,bcuU->acuU", c21, e21)
    tmp = _ein("acuU,ealL->cuUelL", tmp, e24)
    tmp = _ein("cuUelL,LURDQ->cuelRDQ", tmp, np.conj(a2))
    tmp = _ein("cuelRDQ,lurdq->ceRDQrdq", tmp, a2)
    r2 = _ein("ae,fadD->efdD", c24, e23)
    r2 = _ein("efdD,ceRDQrdq->fcRQrq", r2, tmp)
    return _ein("fcRPrp,fcRQrq->PQpq", r1, r2)


def norm_tensor(st, bond, a1q, a2q):
    """``build_norm_tensor`` + ``build_norm_tensor_core`` of the full update
    (acetn/evolution/full_update.py:163-236): the environment of bond
    (s1, s2, k) contracted with the reduced site tensors a1q (r,d,u,y) and
    a2q (d,l,u,x) into n12[y,x,Y,X].  ``build_norm_tensor_core_blocked``
    (full_update.py:239-268) computes the same sum in blocks of the bra legs."""
    s1, s2, k = bond
    t1, t2 = st[s1], st[s2]
    c12 = t1["C"][(k + 1) % 4]; e12 = t1["E"][(k + 1) % 4]; e11 = t1["E"][k % 4]
    c13 = t1["C"][(k + 2) % 4]; e13 = t1["E"][(k + 2) % 4]
    c21 = t2["C"][k % 4]; e21 = t2["E"][k % 4]; e24 = t2["E"][(k + 3) % 4]
    c24 = t2["C"][(k + 3) % 4]; e23 = t2["E"][(k + 2) % 4]
    tmp = _ein("ab,bcrR->acrR", c12, e12)
    tmp = _ein("acrR,eauU->crReuU", tmp, e11)
    tmp = _ein("crReuU,RDUY->creuDY", tmp, np.conj(a1q))
    tmp = _ein("creuDY,rduy->ceDYdy", tmp, a1q)
    n1 = _ein("ab,bfdD->afdD", c13, e13)
    n1 = _ein("afdD,aeDYdy->feYy", n1, tmp)
    tmp = _ein("ab,bcuU->acuU", c21, e21)
    tmp = _ein("acuU,ealL->cuUelL", tmp, e24)
    tmp = _ein("cuUelL,DLUX->cuelXD", tmp, np.conj(a2q))
    tmp = _ein("cuelXD,dlux->ceXDxd", tmp, a2q)
    n2 = _ein("ab,fadD->bfdD", c24, e23)
    n2 = _ein("bfdD,cbXDxd->fcXx", n2, tmp)
    return _ein("fcYy,fcXx->yxYX", n1, n2)


def als_initialize(a12g, shape):
    """``ALSSolver.initialize_reduced_tensors`` (acetn/evolution/
    als_solver.py:120-147): truncated SVD of a12g[(y,p)][(x,q)] to bD
    values, each factor scaled by sqrt(S / S_0)."""
    nD, bD, pD = shape
    m = a12g.transpose(0, 2, 1, 3).reshape(nD * pD, nD * pD)
    u, sv, vh = np.linalg.svd(m)
    sq = np.sqrt(sv[:bD] / sv[0])
    a1r = _ein("ypu,u->yup", u[:, :bD].reshape(nD, pD, bD), sq)
    a2r = _ein("xqv,v->xvq", vh.T[:, :bD].reshape(nD, pD, bD), sq)
    return a1r, a2r


def als_cost(a1r, a2r, a12g, n12):
    """``ALSSolver.calculate_cost`` (als_solver.py:253-262): the distance
    <a12n|N|a12n> - 2 <a12n|N|a12g> up to a constant."""
    a12n = _ein("yup,xuq->yxpq", a1r, a2r)
    d2 = _ein("YXpq,YXpq->", _ein("yxYX,yxpq->YXpq", n12, a12n), a12n)
    d3 = _ein("YXpq,YXpq->", _ein("yxYX,yxpq->YXpq", n12, a12g), a12n)
    return float(d2 - 2.0 * d3)


def _als_solve_ar(r, sm, method, eps):
    """``ALSSolver.solve_ar`` (als_solver.py:212-243): R symmetrised; the
    Cholesky of R + eps max|R| I with two triangular solves (a plain solve of
    the shifted R when the factorisation fails), or the Hermitian
    pseudo-inverse with cutoff eps."""
    nD, bD, pD = sm.shape
    sm = sm.reshape(nD * bD, pD)
    r = r.reshape(nD * bD, nD * bD)
    r = 0.5 * (r + r.T)
    if method == "cholesky":
        r = r + eps * np.abs(r).max() * np.eye(r.shape[0])
        try:
            low = np.linalg.cholesky(r)
            y = np.linalg.solve(low, sm)  # triangular systems, solved densely
            ar = np.linalg.solve(low.T, y)
        except np.linalg.LinAlgError:
            ar = np.linalg.solve(r, sm)
    else:
        ar = np.linalg.pinv(r, rcond=eps, hermitian=True) @ sm
    return ar.reshape(nD, bD, pD)


def als_solve(n12, a12g, shape, niter=100, tol=1e-15, method="cholesky", eps=1e-12):
    """``ALSSolver.solve`` / ``solve_torch`` (als_solver.py:35-82): alternate
    the least-squares updates of a1r (build_s1/build_r1, als_solver.py:
    245-251) and a2r (build_s2/build_r2) until the relative change of the
    cost falls below tol after the second iteration.  Returns (a1r, a2r,
    iterations run)."""
    a1r, a2r = als_initialize(a12g, shape)
    n12g = _ein("yxYX,yxpq->YXpq", n12, a12g)
    d1 = abs(als_cost(a1r, a2r, a12g, n12))
    for i in range(niter):
        s1 = _ein("YXpQ,XUQ->YUp", n12g, a2r)
        r1 = _ein("yYXuQ,XUQ->YUyu", _ein("yxYX,xuq->yYXuq", n12, a2r), a2r)
        a1r = _als_solve_ar(r1, s1, method, eps)
        s2 = _ein("YXPq,YVP->XVq", n12g, a1r)
        r2 = _ein("xYXvP,YVP->XVxv", _ein("yxYX,yvp->xYXvp", n12, a1r), a1r)
        a2r = _als_solve_ar(r2, s2, method, eps)
        d2 = als_cost(a1r, a2r, a12g, n12)
        if abs(d2 - d1) / abs(d1) < tol and i > 1:
            return a1r, a2r, i + 1
        d1 = d2
    return a1r, a2r, niter


def build_site_list(nx, ny):
    """``TensorNetwork.build_site_list`` (acetn/ipeps/tensor_network.py:179-193)."""
    return [(xi, yi) for xi in range(nx) for yi in range(ny)]


def build_bond_list(nx, ny):
    """``TensorNetwork.build_bond_list`` (acetn/ipeps/tensor_network.py:153-177):
    horizontal bonds (k=2) then vertical bonds (k=1)."""
    bonds = []
    for xi in range(nx):
        for yi in range(ny):
            bonds.append(((xi, yi), ((xi + 1) % nx, yi), 2))
    for yi in range(ny):
        for xi in range(nx):
            bonds.append(((xi, yi), (xi, (yi + 1) % ny), 1))
    return bonds


_X = np.array([[0.0, 1.0], [1.0, 0.0]])
_Yr = np.array([[0.0, -1.0], [1.0, 0.0]])
_Z = np.array([[1.0, 0.0], [0.0, -1.0]])


def heisenberg_model(J=1.0):
    """``HeisenbergModel`` (acetn/model/models/heisenberg.py:4-26): bond term
    0.25 J (XX + YY + ZZ) with the real Y convention of
    acetn/model/pauli_matrix.py (YY of two real Y's carries phase -1);
    staggered one-site observables sx, sz."""
    h2 = 0.25 * J * (np.kron(_X, _X) - np.kron(_Yr, _Yr) + np.kron(_Z, _Z))

    def one_site_obs(site):
        sgn = 1.0 if (site[0] + site[1]) % 2 == 0 else -1.0
        return {"sx": sgn * _X, "sz": sgn * _Z}

    return {"one_site_ham": lambda site: None, "two_site_ham": lambda bond: h2,
            "one_site_obs": one_site_obs, "two_site_obs": lambda bond: {}, "dim": 2}


def ising_model(jz=1.0, hx=3.0):
    """``IsingModel`` (acetn/model/models/ising.py:4-21): -jz ZZ on bonds,
    -hx X on sites; one-site observables sx, sz."""
    h2 = -jz * np.kron(_Z, _Z)
    h1 = -hx * _X
    return {"one_site_ham": lambda site: h1, "two_site_ham": lambda bond: h2,
            "one_site_obs": lambda site: {"sx": _X, "sz": _Z},
            "two_site_obs": lambda bond: {}, "dim": 2}


def measure(st, model):
    """``measure`` (acetn/measurement/measure.py:5-28, 114-198): energy per site
    and averaged one-site observables from trace-normalised RDMs.  Also returns
    the per-site and per-bond terms under 'site_terms' / 'bond_terms'."""
    d = model["dim"]
    sites = build_site_list(st.nx, st.ny)
    bonds = build_bond_list(st.nx, st.ny)
    out = {"Energy": 0.0}
    keys = list(model["one_site_obs"]((0, 0)).keys())
    for key in keys:
        out[key] = 0.0
    site_terms, bond_terms = {}, {}
    for s in sites:
        r = site_rdm(st[s])
        norm = np.real(np.trace(r))
        h1 = model["one_site_ham"](s)
        e = 0.0 if h1 is None else np.real(_ein("Pp,pP->", r, h1)) / norm
        site_terms[s] = e
        out["Energy"] += e
        for key, op in model["one_site_obs"](s).items():
            out[key] += np.real(_ein("Pp,pP->", r, op)) / norm
    for key in keys:
        out[key] /= len(sites)
    for s1, s2, k in bonds:
        r = bond_rdm(st, s1, s2, k)
        norm = np.real(_ein("pqpq->", r))
        h2 = model["two_site_ham"]((s1, s2, k)).reshape((d,) * 4)
        e = np.real(_ein("PQpq,pqPQ->", r, h2)) / norm
        bond_terms[(s1, s2, k)] = e
        out["Energy"] += e
    out["Energy"] /= len(sites)
    out["site_terms"] = site_terms
    out["bond_terms"] = bond_terms
    return out
