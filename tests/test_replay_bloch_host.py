"""Host-side checks of the Bloch replay's inputs (no GPU): per-compartment rate lists must cover
every compartment id the walk holds, and a field callable is called on position arrays only when
it takes them."""
import numpy as np
import pytest

from dmipy_sim_gb300 import trajectories as T


def test_per_comp_rates_cover_every_compartment():
    comp = np.array([[0, 1, 2], [2, 1, 0]])
    c, t2, t1 = T._per_comp_rates(comp, [0.07, 0.015, 0.06], None, 0.0, 1.0)
    np.testing.assert_allclose(t2, 1.0 / np.array([0.07, 0.015, 0.06]))
    np.testing.assert_allclose(t1, [1.0, 1.0, 1.0])
    assert c.dtype == np.int32
    assert T._per_comp_rates(comp, None, None, 0.0, 0.0) is None


def test_short_per_comp_list_is_an_index_error():
    comp = np.array([[0, 1, 2]])
    with pytest.raises(IndexError, match="T2_per_comp"):
        T._per_comp_rates(comp, [0.07, 0.015], None, 0.0, 0.0)
    with pytest.raises(IndexError, match="T1_per_comp"):
        T._per_comp_rates(comp, None, [1.0], 0.0, 0.0)
    with pytest.raises(IndexError, match="negative"):
        T._per_comp_rates(np.array([[0, -1]]), [0.07, 0.015], None, 0.0, 0.0)
    with pytest.raises(ValueError, match="comp_traj"):
        T._per_comp_rates(None, [0.07], None, 0.0, 0.0)


def test_field_callable_probe():
    assert T._takes_position_arrays(lambda r: np.sum(np.asarray(r) ** 2, axis=-1))

    def scalar_only(r):
        x, y, z = r            # a (2, 3) array does not unpack into three values
        return x * y * z

    assert not T._takes_position_arrays(scalar_only)

    def broken(r):
        raise RuntimeError("a fault of the provider")

    with pytest.raises(RuntimeError):
        T._takes_position_arrays(broken)
