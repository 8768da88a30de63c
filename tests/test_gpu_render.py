"""GPU parity of the renderer's voxel pack (render.py:176-205 pack_volume_lm, with the shock
proxy inline) and its [1 4 1] prefilter (render.py:281-298), through libnebula's C ABI.  Both
library builds pack with exact code generation (the voxels are a texture format): bit-identical
to the reference kernels, and to the oracle at 128^3."""
import numpy as np
import pytest

from conftest import golden

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

KEYS = ("c_ha", "c_o3", "c_s2", "c_dg", "c_sh", "gs", "ambient", "edge", "inv_L", "dx")


def params(a):
    a = [float(v) for v in a]
    return {"c_ha": a[0:3], "c_o3": a[3:6], "c_s2": a[6:9], "c_dg": a[9:12], "c_sh": a[12:15], "gs": a[15],
            "ambient": a[16], "edge": a[17], "inv_L": a[18:21], "dx": a[21]}


@pytest.fixture(scope="module")
def S():
    from nebulaviewer_gb300 import build
    build.build(verbose=False)
    from nebulaviewer_gb300 import sim
    assert torch.cuda.is_available()
    return sim


@pytest.mark.parametrize("arith", ("exact", "fast"))
@pytest.mark.parametrize("tag", ("jwst", "sho", "nat"))
def test_render_pack_bit_identical_to_reference(S, tag, arith):
    z = golden("render.npz")
    shape = z["p_rho"].shape
    s = S.Sim.from_state(shape, float(z["p_dx"]), z["p_rho"], [], [], [], [], dict(ci_over_cn=12.0),
                         mom=list(z["p_mom"]), rays=(8, 16), fuv_grid=(4, 4, 8), start_main=False, arith=arith)
    s._xi.copy_(torch.as_tensor(z["p_xi"], device="cuda"))
    s._dfront.copy_(torch.as_tensor(z["p_df"], device="cuda"))
    s._g0.copy_(torch.as_tensor(z["p_g0"], device="cuda"))
    pp = z[f"p_{tag}_params"]
    for smooth, ref in ((False, z[f"p_{tag}_packed"]), (True, z[f"p_{tag}_smooth"])):
        out = s.render_pack(params(pp), shock_on=bool(pp[22]), smooth=smooth)
        torch.cuda.synchronize()
        got = out.numpy()
        assert got.shape == shape + (4,) and got.dtype == np.float16
        assert np.array_equal(got.view(np.uint16), ref.view(np.uint16)), (tag, smooth)
    s.close()


def test_render_pack_128_against_oracle(S):
    """a stepped sheet at 128^3 (fronts, FUV, shocks present): bit-identical to the oracle"""
    import oracle as O
    s = S.Sim("sheet", res=128, verbose=False)
    s.step(6)
    s.update_render_fields(force=True)
    z = golden("render.npz")
    pp = params(z["p_jwst_params"])
    pp["inv_L"] = [1.0 / v for v in s.L]
    pp["dx"] = s.dx
    out = s.render_pack(pp, smooth=True).numpy()
    ref = O.render_pack(s.rho.numpy(), [s.mx.numpy(), s.my.numpy(), s.mz.numpy()], s.xi.numpy(), s.dfront.numpy(),
                        s.g0.numpy(), [v for k in KEYS for v in (pp[k] if isinstance(pp[k], list) else [pp[k]])], 1)
    assert np.array_equal(out.view(np.uint16), ref.view(np.uint16))
    assert float((out[..., 3].astype(np.float32) > 0).mean()) > 0.5
    s.close()
