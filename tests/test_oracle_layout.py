"""The oracle's restatement of the coupler's layout transforms
(code/x86/TradDA/DA/EnDNN/src/data_trans.F90:1-70) against numpy index maps."""
import numpy as np

from oracle import oracle as O


def test_atm2endnn_places_a_variable_group():
    rng = np.random.default_rng(1)
    n, nx, ny, ens, n_max, ens_max = 3, 5, 7, 4, 9, 6
    xb = rng.standard_normal((n, nx, ny, ens))
    xb2 = O.struct_atm2endnn(xb, ens_max, n_max, ens_start=2, n_start=4)
    ref = np.zeros((ny, nx, n_max, ens_max))
    ref[:, :, 3:6, 1:5] = np.transpose(xb, (2, 1, 0, 3))
    assert np.array_equal(xb2, ref)
    back = O.struct_endnn2atm(xb2, ens, n, ens_start=2, n_start=4)
    assert np.array_equal(back, xb)


def test_mean_forms():
    rng = np.random.default_rng(2)
    n, nx, ny, n_max = 2, 4, 6, 5
    axb = rng.standard_normal((n, nx, ny))
    axb2 = O.struct_atm2endnn_a(axb, n_max, n_start=3)
    ref = np.zeros((ny, nx, n_max))
    ref[:, :, 2:4] = np.transpose(axb, (2, 1, 0))
    assert np.array_equal(axb2, ref)
    assert np.array_equal(O.struct_endnn2atm_a(axb2, n, n_start=3), axb)
