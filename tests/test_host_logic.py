"""Host-side logic of the package (no GPU): configuration, move order,
site/bond bookkeeping and the state container."""

import pytest
import torch

import acetn_gb300 as gb
from oracle import ctm_oracle as orc


def test_sweep_order_matches_reference_loop():
    for nx, ny in [(2, 2), (3, 2), (2, 4)]:
        assert gb.sweep_order(nx, ny) == orc.sweep_order(nx, ny)


def test_site_and_bond_lists():
    st = gb.IpepsState(2, 3, {"phys": 2, "bond": 2, "chi": 4}, device="cpu")
    assert st.site_list == orc.build_site_list(2, 3)
    assert [tuple(b) for b in st.bond_list] == orc.build_bond_list(2, 3)


def test_config_defaults_and_validation():
    cfg = gb.CTMRGConfig()
    assert (cfg.steps, cfg.projectors, cfg.svd_type, cfg.svd_cutoff, cfg.rsvd_niter,
            cfg.rsvd_oversampling) == (40, "half-system", "rsvd", 1e-12, 2, 2)
    with pytest.raises(ValueError):
        gb.ProjectorCalculator({"projectors": "quarter-system"})
    with pytest.raises(TypeError):
        gb.config.resolve({"no_such_field": 1})
    pc = gb.ProjectorCalculator({"projectors": "full-system"})
    assert pc.calculate == pc.calculate_full_system


def test_reference_style_config_object_is_accepted():
    class RefCfg:
        steps = 3
        projectors = "half-system"
        svd_type = "full-rank"
        svd_cutoff = 1e-10
        rsvd_niter = 1
        rsvd_oversampling = 4
        disable_progressbar = True
    cfg = gb.config.resolve(RefCfg())
    assert cfg.svd_type == "full-rank" and cfg.rsvd_oversampling == 4 and cfg.precision == "fp64"


def test_unknown_site_raises_value_error():
    st = gb.IpepsState(2, 2, {"phys": 2, "bond": 2, "chi": 4}, device="cpu")
    with pytest.raises(ValueError):
        st[(3, 3)]


def test_state_checkpoint_round_trip(tmp_path):
    st = orc.random_state(2, 4, seed=3)
    g = gb.IpepsState.from_arrays(st.sites, 2, 2, 4, device="cpu")
    g.save(tmp_path / "s.pt")
    h = gb.IpepsState.load(tmp_path / "s.pt", device="cpu")
    for s in st.sites:
        assert torch.equal(g[s]["A"], h[s]["A"])
        for k in range(4):
            assert torch.equal(g[s]["E"][k], h[s]["E"][k])


def test_models_match_oracle_hamiltonians():
    import numpy as np
    h = gb.HeisenbergModel(1.0).two_site_hamiltonian(None).numpy()
    assert np.allclose(h, orc.heisenberg_model(1.0)["two_site_ham"](None))
    m = gb.IsingModel(1.0, 3.0)
    assert np.allclose(m.two_site_hamiltonian(None).numpy(), orc.ising_model(1.0, 3.0)["two_site_ham"](None))
    assert np.allclose(m.one_site_hamiltonian((0, 0)).numpy(), -3.0 * np.array([[0, 1], [1, 0]]))


def test_clock_sampler_keeps_samples_of_the_timed_window():
    """bench.py's clock record: only samples that arrived inside the timed
    window count; throttle reasons are collected from them."""
    import importlib.util
    import os
    spec = importlib.util.spec_from_file_location(
        "bench_mod", os.path.join(os.path.dirname(os.path.dirname(__file__)), "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)

    class FakeProc:
        def terminate(self):
            pass

        def wait(self, timeout=None):
            return 0

    s = bench.ClockSampler(0)
    s.proc = FakeProc()
    row = "0, {sm}, 2070, 900.0, 0x0, Not Active, Not Active, {th}, Not Active"
    s.lines = [(0.0, row.format(sm=1000, th="Active")),     # before the window
               (1.00, row.format(sm=2070, th="Not Active")),
               (1.02, row.format(sm=2050, th="Not Active")),
               (9.0, row.format(sm=500, th="Active"))]     # after the window
    s.t0, s.t1 = 0.99, 1.01
    out = s.stop()
    assert out["samples"] == 2 and out["sm_mhz"] == 2060.0 and out["in_window"]
    assert out["reasons"] == [] and out["sm_max_mhz"] == 2070.0
    # a window shorter than the interval keeps the nearest sample
    s.lines = [(0.0, row.format(sm=1000, th="Not Active")), (5.0, row.format(sm=1500, th="Active"))]
    s.t0, s.t1 = 4.9, 4.91
    out = s.stop()
    assert out["samples"] == 1 and out["sm_mhz"] == 1500.0 and not out["in_window"]
    assert out["reasons"] == ["sw_thermal_slowdown"]


def test_reads_a_checkpoint_written_by_the_reference(tmp_path):
    """tests/golden/ref_checkpoint_d2.pt was written by the reference's own
    TensorNetwork.save (tests/golden/make_checkpoint.py); it is read without
    the reference, tensor for tensor, and round-trips through the plain
    checkpoint format."""
    import os
    import numpy as np
    golden = os.path.join(os.path.dirname(__file__), "golden")
    st = gb.IpepsState.load_reference(os.path.join(golden, "ref_checkpoint_d2.pt"), device="cpu")
    z = np.load(os.path.join(golden, "ref_checkpoint_d2.npz"))
    assert (st.nx, st.ny) == (2, 2) and st.dims == {"phys": 2, "bond": 2, "chi": 6}
    for s in st.site_list:
        key = f"{s[0]}_{s[1]}"
        assert np.array_equal(st[s]["A"].numpy(), z[f"{key}_A"])
        for k in range(4):
            assert np.array_equal(st[s]["C"][k].numpy(), z[f"{key}_C{k}"])
            assert np.array_equal(st[s]["E"][k].numpy(), z[f"{key}_E{k}"])
    plain = tmp_path / "plain.pt"
    st.save(plain)
    back = gb.IpepsState.load(plain, device="cpu")
    for s in st.site_list:
        assert torch.equal(back[s]["A"], st[s]["A"])
        assert all(torch.equal(a, b) for a, b in zip(back[s]["E"], st[s]["E"]))
    # a plain checkpoint is not a reference checkpoint
    with pytest.raises(ValueError):
        gb.IpepsState.load_reference(plain, device="cpu")
