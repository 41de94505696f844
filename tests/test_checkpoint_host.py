"""The host side of checkpoint archives, without a GPU: the scenario's
parameter structs and grid survive the archive byte for byte, for every fault
law and with plasticity, and the archive reader rebuilds a scenario whose
derived constants equal the original's."""
import numpy as np
import pytest

from tetemoko_gb300 import _capi as A, checkpoint, scenarios as S

SCENARIOS = {
    "rate_state_slip_law": lambda: S.rate_state(nx=32, ny=16, dx=0.05, state_law=A.TMK_RS_SLIP_LAW),
    "slip_weakening_plastic": lambda: S.slip_weakening(nx=24, ny=12, dx=0.1, plasticity=True),
    "no_fault": lambda: S.Scenario(name="plane", nx=8, ny=8, dx=0.2, cfl=0.5, elastic=S._elastic(),
                                   scheme=S._scheme(A.TMK_FAULT_NONE, bc=(0, 1, 0, 0, 1, 1))),
}


@pytest.mark.parametrize("name", list(SCENARIOS))
def test_scenario_round_trips_through_an_archive(name, tmp_path):
    sc = SCENARIOS[name]()
    path = str(tmp_path / "scenario.npz")
    np.savez(path, **checkpoint._scenario_arrays(sc))
    with np.load(path) as z:
        back = checkpoint._scenario_from(z)
    assert (back.name, back.nx, back.ny, back.dx, back.cfl) == (sc.name, sc.nx, sc.ny, sc.dx, sc.cfl)
    for field in ("elastic", "scheme", "rs", "sw", "plastic"):
        a, b = getattr(sc, field), getattr(back, field)
        assert (a is None) == (b is None), field
        if a is not None:
            assert bytes(a) == bytes(b), field
    assert back.constants() == sc.constants()
    np.testing.assert_array_equal(back.initial_U(), sc.initial_U())
    if sc.scheme.fault_law != A.TMK_FAULT_NONE:
        np.testing.assert_array_equal(back.initial_B(), sc.initial_B())


def test_3d_level_refuses_fabs_of_another_shape_or_type():
    """LinElastLevelGodunov3D copies whole FABs of patch_shapes(p) through the
    library: arrays of another shape, type or layout are refused on the host
    before any copy (checked here without a device level)."""
    from tetemoko_gb300.level import LinElastLevelGodunov3D

    class _Ctx:
        sc = S.rate_state(nx=12, ny=10, dx=0.1)

    lv = LinElastLevelGodunov3D.__new__(LinElastLevelGodunov3D)
    lv.ctx, lv.boxes, lv.domain = _Ctx(), [((0, 0, 0), (5, 4, 3))], ((0, 0, 0), (11, 9, 7))
    ushape, bshape = lv.patch_shapes(0)
    assert ushape == (22, 12, 13, 14) and bshape == (_Ctx.sc.nbdry, 12, 14)
    lv._checked(0, np.zeros(ushape), np.zeros(bshape), True)
    for U, B in ((np.zeros((22, 12, 13, 13)), None), (np.zeros(ushape, dtype=np.float32), None),
                 (np.zeros(ushape[::-1]).T, None), (np.zeros(ushape), np.zeros((11, 12, 13)))):
        with pytest.raises(ValueError):
            lv._checked(0, U, B, True)
