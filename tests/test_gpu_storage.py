"""Float32 site storage (the batched TFIM configuration stores float32 and
computes projectors in FP64): the library widens on entry, the moves write
float32 back, and results agree with float64 storage to float32 rounding."""

import pytest
import torch

import acetn_gb300 as gb

pytestmark = pytest.mark.gpu

CFG = dict(projectors="half-system", svd_type="full-rank", disable_progressbar=True)


def _copy(st, dtype):
    g = gb.IpepsState(st.nx, st.ny, st.dims, st.device)
    for s in st.site_list:
        v = st[s]
        g[s] = {"A": v["A"].to(dtype), "C": [c.to(dtype) for c in v["C"]],
                "E": [e.to(dtype) for e in v["E"]]}
    return g


def test_float32_storage_matches_float64_storage():
    st = gb.random_state(3, 12, 11, device="cuda")
    gb.ctmrg(st, gb.CTMRGConfig(**CFG, steps=2))
    s64, s32 = _copy(st, torch.float64), _copy(st, torch.float32)
    for state in (s64, s32):
        mv = gb.DirectionalMover(gb.CTMRGConfig(**CFG))
        for k in range(4):
            mv.move(state, k, 0)
    for s in s32.site_list:
        assert all(t.dtype == torch.float32 for t in s32[s]["C"] + s32[s]["E"])
    model = gb.HeisenbergModel(1.0)
    e64 = float(gb.measure(s64, model, verbose=False)["Energy"])
    e32 = float(gb.measure(s32, model, verbose=False)["Energy"])
    assert abs(e32 - e64) <= 1e-5 * abs(e64), (e32, e64)


def test_float16_storage_is_rejected():
    st = _copy(gb.random_state(2, 4, 1, device="cuda"), torch.float16)
    with pytest.raises(ValueError):
        gb.DirectionalMover(gb.CTMRGConfig(**CFG)).move(st, 0, 0)
