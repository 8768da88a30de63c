"""Snapshot and frame formats: the 13 B/cell timeline snapshot (timeline.py:19-89) and the bake
frame (bake.py:95-102) with the shock proxy (nebula3d.py:182-191), byte-exact against the
reference's kernels (golden fixtures) and its numpy expressions; Timeline capture / restore /
branch."""
import numpy as np
import pytest

from conftest import golden

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S():
    from nebulaviewer_gb300 import build
    build.build(verbose=False)
    from nebulaviewer_gb300 import sim
    return sim


def sim_with(S, d, fp32):
    shape = d["t_rho"].shape
    P = dict(fp32_fields=fp32)
    s = S.Sim.from_state(shape, 0.125, d["t_rho"], [], [], [], [], P, mom=list(d["t_mom"]), rays=(8, 16),
                         fuv_grid=(4, 4, 8), start_main=False)
    s._xi.copy_(torch.as_tensor(d["t_xi"]))
    s._dfront.copy_(torch.as_tensor(d["t_df32" if fp32 else "t_df16"]))
    s._g0.copy_(torch.as_tensor(d["t_g032" if fp32 else "t_g016"]))
    return s


@pytest.mark.parametrize("tag,fp32", (("lm", False), ("f32", True)))
def test_snapshot_pack_unpack_match_reference(S, tag, fp32):
    d = golden("timeline.npz")
    s = sim_with(S, d, fp32)
    n = s._n
    buf = torch.zeros(13 * n, dtype=torch.uint8, device="cuda")
    s.snapshot_pack(buf)
    torch.cuda.synchronize()
    b = buf.cpu().numpy()
    planes = {"r": (0, 2), "mx": (2 * n, 2), "my": (4 * n, 2), "mz": (6 * n, 2), "xi": (8 * n, 1), "df": (9 * n, 2),
              "g0": (11 * n, 2)}
    for k, (off, w) in planes.items():
        got = b[off:off + w * n]
        ref = d[f"t_{tag}_pack_{k}"].reshape(-1).view(np.uint8)
        assert np.array_equal(got, ref), k
    s.snapshot_unpack(buf)
    torch.cuda.synchronize()
    for k, attr in (("rho", "_rho"), ("mx", "_mx"), ("my", "_my"), ("mz", "_mz"), ("xi", "_xi"), ("df", "_dfront"),
                    ("g0", "_g0")):
        got = getattr(s, attr).cpu().numpy()
        ref = d[f"t_{tag}_unpack_{k}"]
        assert np.array_equal(got.view(np.uint8), ref.astype(got.dtype).view(np.uint8)), k
    s.close()


def test_bake_frame_matches_reference_expressions(S):
    d = golden("timeline.npz")
    for fp32 in (False, True):
        s = sim_with(S, d, fp32)
        s._rho.copy_(torch.as_tensor(d["t_shock_rho"]))
        fr = s.frame()
        rho, xi, df, g0 = (t.cpu().numpy() for t in (s._rho, s._xi, s._dfront, s._g0))
        sh = s.shock.numpy()
        # bake.py:95-102, verbatim numpy
        ref = dict(g0=np.minimum(g0, 6e4).astype(np.float16), rho=rho.astype(np.float16),
                   xi=np.round(np.clip(xi, 0, 1) * 255).astype(np.uint8),
                   df=np.clip(df, -4, 4).astype(np.float16), sh=np.minimum(sh, 6e4).astype(np.float16))
        for k in ref:
            assert np.array_equal(fr[k].view(np.uint8), ref[k].view(np.uint8)), (k, fp32)
        s.close()
    s = sim_with(S, d, False)
    s._rho.copy_(torch.as_tensor(d["t_shock_rho"]))
    assert np.array_equal(s.shock.numpy().view(np.uint32), d["t_shock"].view(np.uint32))
    s.close()


def test_timeline_capture_restore_branch(S):
    from nebulaviewer_gb300 import ics
    from nebulaviewer_gb300.timeline import Timeline
    ic = ics.torus(seed=9, device="cuda", shape=(32, 32, 32), nstars=2)
    s = S.Sim.from_state(ic["shape"], ic["dx"], ic["rho"], ic["stars"], ic["kinds"], ic["jets"], ic["jkinds"],
                         dict(ic["P"], t_end=0.004), rays=(64, 128), fuv_grid=(16, 16, 32))
    tl = Timeline(budget_gb=32 * 32 * 32 * 13 * 4 / 1e9)          # room for 4 snapshots
    tl.clear(s)
    for _ in range(12):
        s.step(1)
        tl.maybe_capture(s)
    assert 1 <= len(tl.snaps) <= tl.capacity() == 4
    i = len(tl.snaps) // 2
    tau = tl.snaps[i]["tau"]
    outs = []
    for _ in range(2):                       # restore twice, step the same way: identical results
        assert tl.restore(s, i)
        assert s.tau() == tau
        buf = tl.snaps[i]["buf"]
        s.step(3)
        outs.append([t.clone() for t in (s._rho, s._mx, s._xi)] + [s.t])
    for a, b in zip(outs[0][:3], outs[1][:3]):
        assert torch.equal(a, b)
    assert outs[0][3] == outs[1][3]
    tl.truncate_after(tau)
    assert all(x <= tau + 1e-12 for x in tl.taus())
    assert "snapshots" in tl.status()
    s.close()
