"""The drop-in's hand-over from a reference instance refuses what this package leaves out before
touching the device: a cropped window (crop.py; the reference sets L_full, sim.py:634).  No GPU."""
import types

import pytest

pytest.importorskip("torch")
S = pytest.importorskip("nebulaviewer_gb300.sim")


def test_a_cropped_reference_instance_is_refused():
    ref = types.SimpleNamespace(L_full=(3.0, 1.5, 1.5), crop_origin=(0.5, 0.0, 0.0), P={"trigger": 0.0})
    with pytest.raises(NotImplementedError, match="cropped"):
        S.Sim.from_reference(ref)
