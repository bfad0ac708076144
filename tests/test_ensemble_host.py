"""CPU checks of the ensemble's host-side sizing (no device needed)."""
import pytest


@pytest.mark.parametrize("n,groups,fits", [(256, 8, True), (256, 4, False), (192, 4, True), (192, 2, False),
                                           (128, 2, True), (128, 1, False), (96, 1, True), (64, 1, True)])
def test_shared_memory_budget(fen_lib, n, groups, fits):
    import fen_gb300 as F

    b = F.ensemble_smem_bytes(n, groups)
    assert b > 0
    assert (b <= 232448) == fits


def test_invalid_tile_rejected(fen_lib):
    import fen_gb300 as F

    assert F.ensemble_smem_bytes(96, 5) == 0
    assert F.ensemble_smem_bytes(0, 1) == 0
