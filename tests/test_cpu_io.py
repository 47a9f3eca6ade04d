"""Snapshot files in the reference's layout (field.py:83-173, rbc2d_base.py:208-228), host side."""
import numpy as np

from pypde_gb300 import io


def test_snapshot_names_follow_the_reference():
    assert io.snapshot_name(1.5, None, "flow", True) == "flow_0001.50.h5"
    assert io.snapshot_name(12.345, None, "", True) == "_0012.35.h5"
    assert io.snapshot_name(3.0, None, "flow", False) == "flow.h5"
    assert io.snapshot_name(3.0, "given.h5") == "given.h5"


def test_store_round_trip_and_overwrite(tmp_path):
    name = str(tmp_path / "snap.h5")
    rng = np.random.default_rng(0)
    a, b = rng.standard_normal((5, 4)), rng.standard_normal((5, 4))
    with io.Store(name, "a") as st:
        st.write("temp/vhat", a)
        st.write("time", 0.25)
    with io.Store(name, "a") as st:          # an existing dataset is overwritten, others kept
        assert "temp/vhat" in st and "time" in st
        st.write("temp/vhat", b)
        st.write("ra", 1e5)
    with io.Store(name, "r") as st:
        assert np.array_equal(st.read("temp/vhat"), b)
        assert float(st.read("time")) == 0.25 and float(st.read("ra")) == 1e5
    path = io.container_path(name)
    assert path == name if io.h5py is not None else path.endswith("snap.npz")
