"""Host-side pieces of the learned guess (no GPU): the training cells drawn
for the two shipped networks."""
import numpy as np

from dftpy_gb300 import systems


def _guess_module():
    import importlib
    return importlib.import_module("dftpy_gb300.guess")


def test_training_cells_pure_al_and_jitter():
    G = _guess_module()
    ideal = systems.fcc_supercell((2, 2, 2), sigma=0.0, seed=0, nr=(64, 64, 64))
    for seed, sigma in ((1000, 0.1), (1001, 0.15), (1002, 0.1)):
        st = G.training_cell(seed, mg_max=0.0, sigmas=(0.1, 0.15))
        assert set(st.symbols) == {"Al"} and st.nat == 32 and tuple(st.nr) == (64, 64, 64)
        # the jitter is the fcc_supercell draw with this cell's sigma
        ref = systems.fcc_supercell((2, 2, 2), sigma=sigma, seed=seed, nr=(64, 64, 64))
        np.testing.assert_allclose(st.positions, ref.positions, rtol=0, atol=1e-12)
        d = np.asarray(st.positions) - np.asarray(ideal.positions)
        assert 0.3 * sigma < np.sqrt((d ** 2).mean()) < 3.0 * sigma


def test_training_cells_alloy_default():
    G = _guess_module()
    mg = [G.training_cell(s).symbols.count("Mg") for s in range(1000, 1016)]
    assert max(mg) > 0 and min(mg) >= 0 and max(mg) <= 0.6 * 32
