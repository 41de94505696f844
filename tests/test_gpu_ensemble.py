"""Ensembles: independent scenarios with their own friction, prestress and
grids stepped as one level give, scenario by scenario, exactly what a level of
that scenario alone gives (the kernels compute every patch on its own, so the
results are bitwise equal), in FP64 and in the mixed form, call by call and
replayed from a CUDA graph."""
import numpy as np
import pytest

from tetemoko_gb300 import _capi as A, scenarios as S
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu
G = A.TMK_NGHOST

SMALL_GRIDS = ((64, 32), (96, 32), (128, 64))


def tiles(nx, ny, t):
    return [(x, y, min(x + t, nx) - 1, min(y + t, ny) - 1) for y in range(0, ny, t) for x in range(0, nx, t)]


def _members(n, prec, plastic=False):
    out = []
    for k in range(n):
        sc, tau0 = S.ensemble_member(k, precision=prec, grids=SMALL_GRIDS)
        if plastic:
            sc.scheme.plasticity = 1
            sc.plastic = S.plastic_params()
        U, B = S.prestressed_state(sc, tau0)
        out.append((sc, U, B))
    return out


def _run(members, nsteps, tile, graph=False):
    from tetemoko_gb300.level import Context, LinElastEnsemble, LinElastLevelGodunov
    ctxs = [Context(sc) for sc, _, _ in members]
    doms = [(0, 0, sc.nx - 1, sc.ny - 1) for sc, _, _ in members]
    ens = LinElastEnsemble(ctxs, doms, [tiles(sc.nx, sc.ny, tile) for sc, _, _ in members])
    for k, (sc, U, B) in enumerate(members):
        ens.set_scenario(k, U, B)
    dt = members[0][0].dt()
    if graph:
        g = ens.graph(nsteps, 0.0, dt)
        g.launch(0.0)
        g.close()
    else:
        for s in range(nsteps):
            ens.step(s * dt, dt)
    rc, info = ens.status()
    assert rc == 0, info
    res = []
    for k, (sc, U, B) in enumerate(members):
        Uo, Bo = U.copy(), B.copy()
        ens.get_scenario(k, Uo, Bo)
        res.append((Uo, Bo))
    singles = []
    for k, (sc, U, B) in enumerate(members):
        lv = LinElastLevelGodunov(ctxs[k], tiles(sc.nx, sc.ny, tile))
        lv.set_level(U, B)
        for s in range(nsteps):
            lv.step(s * dt, dt)
        Uo, Bo = U.copy(), B.copy()
        lv.get_level(Uo, Bo)
        singles.append((Uo, Bo))
        lv.close()
    ens.close()
    for c in ctxs:
        c.close()
    return res, singles


@pytest.mark.parametrize("prec", [A.TMK_PREC_FP64, A.TMK_PREC_MIXED], ids=["fp64", "mixed"])
def test_ensemble_equals_single_scenarios(cuda_lib, prec):
    members = _members(5, prec)
    assert len({(sc.nx, sc.ny) for sc, _, _ in members}) > 1       # uneven grids in one launch
    assert len({sc.rs.a for sc, _, _ in members}) == 5
    res, singles = _run(members, 8, 32)
    vs = (slice(None), slice(G, -G), slice(G, -G))
    for (Ue, Be), (Us, Bs), (sc, U0, _) in zip(res, singles, members):
        np.testing.assert_array_equal(Ue[vs], Us[vs])
        np.testing.assert_array_equal(Be[:, G:-G], Bs[:, G:-G])
        assert rel_err(Ue[vs], U0[vs]) > 0          # the step did something


def test_ensemble_plastic_equals_single_scenarios(cuda_lib):
    members = _members(3, A.TMK_PREC_MIXED, plastic=True)
    res, singles = _run(members, 6, 32)
    for (Ue, Be), (Us, Bs) in zip(res, singles):
        np.testing.assert_array_equal(Ue[:, G:-G, G:-G], Us[:, G:-G, G:-G])
        np.testing.assert_array_equal(Be[:, G:-G], Bs[:, G:-G])


def test_ensemble_graph_equals_single_scenarios(cuda_lib):
    members = _members(4, A.TMK_PREC_MIXED)
    res, singles = _run(members, 6, 32, graph=True)
    for (Ue, Be), (Us, Bs) in zip(res, singles):
        np.testing.assert_array_equal(Ue[:, G:-G, G:-G], Us[:, G:-G, G:-G])
        assert rel_err(Be[:, G:-G], Bs[:, G:-G]) <= 1e-14     # rupture times: t0 + k dt summed differently


def test_ensemble_descriptor_checks(cuda_lib):
    from tetemoko_gb300.level import Context, LinElastEnsemble, LinElastLevelGodunov
    sa, _ = S.ensemble_member(0, grids=SMALL_GRIDS)
    sb, _ = S.ensemble_member(1, grids=SMALL_GRIDS)
    ca, cb = Context(sa), Context(sb)
    da, db = (0, 0, sa.nx - 1, sa.ny - 1), (0, 0, sb.nx - 1, sb.ny - 1)
    # the scenarios' patches may overlap in index space: they are different domains
    ens = LinElastEnsemble([ca, cb], [da, db], [tiles(sa.nx, sa.ny, 32), tiles(sb.nx, sb.ny, 32)])
    # ensembles do not take coarse-fine coupling
    other = LinElastLevelGodunov(ca, tiles(sa.nx, sa.ny, 32))
    with pytest.raises(A.TmkError):
        ens.attach_coarser(other, 2)
    ens.close()
    other.close()
    # overlapping patches within one scenario
    with pytest.raises(A.TmkError):
        LinElastEnsemble([ca, cb], [da, db], [[(0, 0, 31, 31), (16, 0, 47, 31)], tiles(sb.nx, sb.ny, 32)])
    # a patch outside its scenario's domain
    with pytest.raises(A.TmkError):
        LinElastEnsemble([ca, cb], [da, (0, 0, 31, 31)], [tiles(sa.nx, sa.ny, 32), [(0, 0, 63, 31)]])
    # scenarios must share the bulk parameters
    sc2, _ = S.ensemble_member(2, grids=SMALL_GRIDS)
    sc2.elastic.sxx0 = -5.0
    c2 = Context(sc2)
    with pytest.raises(A.TmkError):
        LinElastEnsemble([ca, c2], [da, (0, 0, sc2.nx - 1, sc2.ny - 1)],
                         [tiles(sa.nx, sa.ny, 32), tiles(sc2.nx, sc2.ny, 32)])
    for c in (ca, cb, c2):
        c.close()
