"""Generate the golden vectors in this directory by running the Ace-TN
reference itself (CPU, float64) on seeded inputs.

Run in a container where the reference source tree is available:

    python tests/golden/make_golden.py /path/to/ace-tn

The reference draws the random test matrices of its randomized SVD with
``torch.randn``; during generation that call is replaced by
``oracle.ctm_oracle.OmegaStream`` so that the oracle and the GPU path can be
fed the same matrices later.  Only gauge-invariant quantities of SVD-dependent
results are stored (singular values, the oblique projector P2 P1^T, RDMs,
energies, corner spectra); quarter tensors do not depend on an SVD and are
stored entry by entry.

The ``toml`` package that the reference imports for logging is replaced by a
small stand-in built on the standard library's ``tomllib``.
"""

import os
import sys
import types
import tomllib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)


def _install_toml_stub():
    mod = types.ModuleType("toml")

    def load(f):
        if isinstance(f, str):
            with open(f, "rb") as fh:
                return tomllib.load(fh)
        return tomllib.load(f)

    mod.load = load
    mod.loads = tomllib.loads
    mod.dumps = lambda d: repr(d) + "\n"
    sys.modules["toml"] = mod


def main(ref_root):
    _install_toml_stub()
    sys.path.insert(0, ref_root)
    import torch
    torch.set_num_threads(8)
    from oracle import ctm_oracle as orc
    from acetn.ipeps import Ipeps
    from acetn.renormalization.directional_mover import DirectionalMover
    from acetn.renormalization.projectors import ProjectorCalculator
    from acetn.measurement.rdm import RDM
    from acetn.ipeps.bond import Bond
    from acetn.model.model_factory import model_factory

    stream = {"s": None}
    real_randn = torch.randn

    def fake_randn(*size, dtype=None, device=None, **kw):
        if stream["s"] is None:
            return real_randn(*size, dtype=dtype, device=device, **kw)
        n, q = size
        return torch.from_numpy(stream["s"](n, q)).to(dtype=dtype or torch.float64)

    torch.randn = fake_randn

    def make_ipeps(D, chi, model, params, ctm):
        cfg = {"dtype": "float64", "device": "cpu",
               "TN": {"nx": 2, "ny": 2, "dims": {"phys": 2, "bond": D, "chi": chi}},
               "model": {"name": model, "params": params},
               "ctmrg": dict(ctm, disable_progressbar=True)}
        return Ipeps(cfg)

    def load_state(ip, st):
        for s in st.sites:
            ip[s]["A"] = torch.from_numpy(st[s]["A"].copy())
            ip[s]["C"] = [torch.from_numpy(c.copy()) for c in st[s]["C"]]
            ip[s]["E"] = [torch.from_numpy(e.copy()) for e in st[s]["E"]]
        ip.site_states_initialized = True

    def dump_state(ip, prefix, out):
        for s in ip.site_list:
            tag = f"{prefix}_{s[0]}{s[1]}"
            out[tag + "_A"] = ip[s]["A"].numpy().copy()
            for k in range(4):
                out[f"{tag}_C{k}"] = ip[s]["C"][k].numpy().copy()
                out[f"{tag}_E{k}"] = ip[s]["E"][k].numpy().copy()

    def spectra(ip, prefix, out):
        for s in ip.site_list:
            for k in range(4):
                c = ip[s]["C"][k].numpy()
                sv = np.linalg.svd(c, compute_uv=False)
                out[f"{prefix}_spec_{s[0]}{s[1]}_C{k}"] = sv / sv[0]

    def rdms(ip, model, prefix, out):
        rdm = RDM(ip)
        for s in ip.site_list:
            r = rdm[s].numpy()
            out[f"{prefix}_site_rdm_{s[0]}{s[1]}"] = r / np.trace(r)
        for b in ip.bond_list:
            r = rdm[b].numpy()
            out[f"{prefix}_bond_rdm_{b.s1[0]}{b.s1[1]}_{b.s2[0]}{b.s2[1]}_{b.k}"] = \
                r / np.einsum("pqpq->", r)
        m = ip.measure(model=model)
        for key, val in m.items():
            out[f"{prefix}_meas_{key}"] = np.array(float(val))

    # ------------------------------------------------------------ 1. small-move case
    # D=3, chi=9 Heisenberg, environment grown by 2 full-rank CTMRG iterations.
    out = {}
    st = orc.random_state(3, 9, seed=11)
    ip = make_ipeps(3, 9, "heisenberg", {"J": 1.0},
                    {"steps": 2, "svd_type": "full-rank", "projectors": "half-system"})
    load_state(ip, st)
    ip.renormalize()
    dump_state(ip, "in", out)
    for k in range(4):
        q, qD = ProjectorCalculator.make_quarter_tensor(ip[(0, 0)], k)
        out[f"quarter_00_k{k}"] = q.numpy().copy()
    # projectors of every direction, four variants, shared Omega stream
    sites_k = {0: [(0, 0), (1, 0), (1, 1), (0, 1)], 1: [(0, 0), (0, 1), (1, 1), (1, 0)],
               2: [(0, 0), (1, 0), (1, 1), (0, 1)], 3: [(0, 0), (0, 1), (1, 1), (1, 0)]}
    for proj in ("half-system", "full-system"):
        for svd_type in ("rsvd", "full-rank"):
            ip.config.ctmrg.projectors = proj
            ip.config.ctmrg.svd_type = svd_type
            ip.config.ctmrg.rsvd_oversampling = 2
            pc = ProjectorCalculator(ip.config.ctmrg)
            for k in range(4):
                stream["s"] = orc.OmegaStream(1000 + k)
                p1, p2 = pc.calculate(ip, sites_k[k], k)
                p1 = p1.numpy(); p2 = p2.numpy()
                n1 = p1.shape[0] * p1.shape[1] * p1.shape[2]
                n2 = p2.shape[0] * p2.shape[1] * p2.shape[2]
                oblique = p2.reshape(n2, -1) @ p1.reshape(n1, -1).T
                tag = f"proj_{proj[:4]}_{svd_type[:4]}_k{k}"
                out[tag + "_oblique"] = oblique
                out[tag + "_chi"] = np.array(p1.shape[-1])
                stream["s"] = None
    # rSVD of the half-system product with a shared Omega
    from acetn.linalg import fused_matmul_svd_lowrank, svd_lowrank, fused_3matmul_svd_lowrank
    q1, _ = ProjectorCalculator.make_quarter_tensor(ip[(0, 0)], 0)
    q4, _ = ProjectorCalculator.make_quarter_tensor(ip[(0, 1)], 3)
    stream["s"] = orc.OmegaStream(77)
    u, s, v = fused_matmul_svd_lowrank(q1, q4, q=11, niter=2)
    out["rsvd_fused_s"] = s.numpy()
    out["rsvd_fused_usv"] = (u @ torch.diag(s) @ v.T).numpy()
    stream["s"] = orc.OmegaStream(78)
    u, s, v = svd_lowrank(q1, q=11, niter=2)
    out["rsvd_plain_s"] = s.numpy()
    out["rsvd_plain_usv"] = (u @ torch.diag(s) @ v.T).numpy()
    q2, _ = ProjectorCalculator.make_quarter_tensor(ip[(1, 0)], 1)
    q3, _ = ProjectorCalculator.make_quarter_tensor(ip[(1, 1)], 2)
    stream["s"] = orc.OmegaStream(79)
    u, s, v = fused_3matmul_svd_lowrank(q2, q1, q4, q3, q=11, niter=2)
    out["rsvd_fused3_s"] = s.numpy()
    out["rsvd_fused3_usv"] = (u @ torch.diag(s) @ v.T).numpy()
    stream["s"] = None
    # one move of each direction (half-system rsvd), gauge-invariant results
    model = model_factory.create(ip.config.model)
    ip.config.ctmrg.projectors = "half-system"
    ip.config.ctmrg.svd_type = "rsvd"
    for k, name in enumerate(("left", "up", "right", "down")):
        base = {}
        dump_state(ip, "tmp", base)
        mover = DirectionalMover(ip.config.ctmrg)
        stream["s"] = orc.OmegaStream(2000 + k)
        getattr(mover, f"{name}_move")(ip, 0)
        stream["s"] = None
        spectra(ip, f"move_{name}", out)
        rdms(ip, model, f"move_{name}", out)
        # restore the input state for the next direction
        for s in ip.site_list:
            tag = f"tmp_{s[0]}{s[1]}"
            ip[s]["C"] = [torch.from_numpy(base[f"{tag}_C{kk}"]) for kk in range(4)]
            ip[s]["E"] = [torch.from_numpy(base[f"{tag}_E{kk}"]) for kk in range(4)]
    rdms(ip, model, "input", out)
    np.savez_compressed(os.path.join(HERE, "move_d3_chi9.npz"), **out)

    # ------------------------------------------------------------ 2. full CTMRG runs
    # Heisenberg J=1, D=2, chi=20, seeded N(0,1) site tensors, 30 iterations.
    for svd_type, fname in (("full-rank", "ctmrg_d2_chi20_fullrank.npz"),
                            ("rsvd", "ctmrg_d2_chi20_rsvd.npz")):
        out = {}
        st = orc.random_state(2, 20, seed=1234)
        ip = make_ipeps(2, 20, "heisenberg", {"J": 1.0},
                        {"steps": 30, "svd_type": svd_type, "projectors": "half-system"})
        load_state(ip, st)
        dump_state(ip, "in", out)
        stream["s"] = orc.OmegaStream(5)
        ip.renormalize()
        stream["s"] = None
        model = model_factory.create(ip.config.model)
        spectra(ip, "out", out)
        rdms(ip, model, "out", out)
        np.savez_compressed(os.path.join(HERE, fname), **out)

    # Transverse-field Ising, D=3, chi=12, full-system full-rank projectors, 10 iterations
    out = {}
    st = orc.random_state(3, 12, seed=99, bias=1e-2)
    ip = make_ipeps(3, 12, "ising", {"jz": 1.0, "hx": 3.0},
                    {"steps": 10, "svd_type": "full-rank", "projectors": "full-system"})
    load_state(ip, st)
    dump_state(ip, "in", out)
    ip.renormalize()
    model = model_factory.create(ip.config.model)
    spectra(ip, "out", out)
    rdms(ip, model, "out", out)
    np.savez_compressed(os.path.join(HERE, "ctmrg_ising_d3_chi12_full.npz"), **out)

    # ------------------------------------------------------------ 3. ground-state fixtures
    gs_dir = os.path.join(ref_root, "tests", "integration", "ipeps_gs")
    inp_dir = os.path.join(ref_root, "tests", "integration", "input")
    energies = {}
    with open(os.path.join(gs_dir, "energies.csv")) as fh:
        for line in fh:
            name, e = line.strip().split(",")
            energies[name] = float(e)
    for case in ("ising_dims_2_20_dtau_001_hx_295", "heisenberg_dims_3_16_dtau_001"):
        import toml
        cfg = toml.load(os.path.join(inp_dir, case + ".toml"))
        cfg.setdefault("ctmrg", {})["disable_progressbar"] = True
        ip = Ipeps(cfg)
        ip.load(os.path.join(gs_dir, case + ".pt"))
        out = {"published_energy": np.array(energies[case])}
        dump_state(ip, "in", out)
        model = model_factory.create(ip.config.model)
        rdms(ip, model, "in", out)
        # five more CTMRG iterations with each SVD type (shared Omega for rsvd)
        for svd_type in ("full-rank", "rsvd"):
            ip2 = Ipeps(cfg)
            ip2.load(os.path.join(gs_dir, case + ".pt"))
            ip2.config.ctmrg.svd_type = svd_type
            ip2.config.ctmrg.steps = 5
            stream["s"] = orc.OmegaStream(31)
            ip2.renormalize()
            stream["s"] = None
            rdms(ip2, model, f"after5_{svd_type[:4]}", out)
            spectra(ip2, f"after5_{svd_type[:4]}", out)
        np.savez_compressed(os.path.join(HERE, f"gs_{case}.npz"), **out)
    torch.randn = real_randn
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
