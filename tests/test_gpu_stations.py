"""Fault and body stations recorded on the device == the reference's
interpolation (AMRLevelLinElast::writeStationLevel) of the level's state after
each step, bit for bit; records in graphs and inside a subcycled hierarchy;
the station files in the reference's format."""
import os

import numpy as np
import pytest

import oracle as O
from tetemoko_gb300 import _capi as A, scenarios as S
from tests import amr_helpers as H
from tests.helpers import perturbed_state

pytestmark = pytest.mark.gpu
G = A.TMK_NGHOST
BOXES = [(0, 0, 20, 9), (21, 0, 63, 9), (0, 10, 31, 31), (32, 10, 63, 31)]
# fault stations: inside a patch, straddling the patch edge at 20|21, at the last face;
# body stations: inside, across the patch corner (31|32, 9|10), and outside the domain
FAULT_X = [1.234, 2.07, 6.36]
BODY_XY = [(0.95, 0.55), (3.2, 1.0), (9.0, 1.0)]


def _setup(prec, kind="rs"):
    from tetemoko_gb300.level import Context, LinElastLevelGodunov
    sc = S.rate_state(nx=64, ny=32, dx=0.1, precision=prec) if kind == "rs" else \
        S.slip_weakening(nx=64, ny=32, dx=0.1, precision=prec)
    Ug = perturbed_state(sc, np.random.default_rng(61), amp_v=0.05, amp_s=1.0)
    Bg = sc.initial_B()
    ctx = Context(sc)
    lvl = LinElastLevelGodunov(ctx, BOXES)
    lvl.set_level(Ug, Bg)
    return sc, ctx, lvl, Ug, Bg


@pytest.mark.parametrize("prec", [A.TMK_PREC_FP64, A.TMK_PREC_MIXED], ids=["fp64", "mixed"])
@pytest.mark.parametrize("kind", ["rs", "sw"])
def test_station_records_match_the_reference_interpolation(cuda_lib, prec, kind):
    from tetemoko_gb300.stations import Stations
    sc, ctx, lvl, Ug, Bg = _setup(prec, kind)
    st = Stations(lvl, FAULT_X, BODY_XY, capacity=16)
    assert st.present == [True, True, True, True, True, False]
    st.attach()
    dt = sc.dt()
    want = []
    for k in range(5):
        lvl.step(k * dt, dt)
        U, B = Ug.copy(), Bg.copy()
        lvl.get_level(U, B)
        want.append(O.station_values((0, 0, 63, 31), sc.dx, U, B, FAULT_X, BODY_XY[:2]))
    rec = st.read()
    assert rec["dropped"] == 0 and len(rec["time"]) == 5
    np.testing.assert_array_equal(rec["time"], [k * dt + dt for k in range(5)])
    for k in range(5):
        np.testing.assert_array_equal(rec["fault"][k], want[k][0])
        np.testing.assert_array_equal(rec["body"][k, :2], want[k][1])
        assert np.isnan(rec["body"][k, 2]).all()
    st.close()
    lvl.close()
    ctx.close()


def test_station_records_in_a_graph_and_when_full(cuda_lib):
    from tetemoko_gb300.stations import Stations
    sc, ctx, lvl, Ug, Bg = _setup(A.TMK_PREC_MIXED)
    st = Stations(lvl, FAULT_X[:1], BODY_XY[:1], capacity=6)
    st.attach()
    dt = sc.dt()
    g = lvl.graph(4, 0.0, dt)
    g.launch(0.0)
    g.launch(4 * dt)
    g.close()
    rec = st.read()
    assert len(rec["time"]) == 6 and rec["dropped"] == 2        # capacity 6, 8 steps
    np.testing.assert_allclose(rec["time"], [(k + 1) * dt for k in range(6)], rtol=1e-14)
    st.detach()
    lvl.step(8 * dt, dt)
    assert len(st.read()["time"]) == 0
    st.record(1.5)
    r = st.read()
    assert r["time"].tolist() == [1.5]
    st.close()
    lvl.close()
    ctx.close()


@pytest.mark.parametrize("r", [2, 4])
def test_stations_in_a_subcycled_hierarchy(cuda_lib, r):
    """The coarse level records after its finer level's substeps, reflux and
    average-down (postTimeStep's order); the fine level after each substep."""
    from tetemoko_gb300.amr import AMRHierarchy
    from tetemoko_gb300.level import Context
    from tetemoko_gb300.stations import Stations
    from tests.test_gpu_amr import _levels_on_gpu, _read
    sc = S.rate_state(nx=64, ny=32, dx=0.1)
    datas = H.hierarchy(sc, np.random.default_rng(62), nlev=2, ratios=(r, r))
    ctx = Context(sc)
    lvs = _levels_on_gpu(ctx, datas)
    h = AMRHierarchy(lvs, [r])
    fx = [3.33]
    sts = [Stations(lv, fx, [(3.21, 0.45)], capacity=8) for lv in lvs]
    for s in sts:
        s.attach()
    dt0 = sc.dt()
    h.step(dt0)
    rc, rf = sts[0].read(), sts[1].read()
    np.testing.assert_allclose(rc["time"], [dt0], rtol=1e-15)
    np.testing.assert_allclose(rf["time"], [dt0 * (k + 1) / r for k in range(r)], rtol=1e-15)
    d0 = _read(lvs[0], datas[0])
    Ug = np.zeros((22, 32 + 2 * G, 64 + 2 * G))
    Bg = np.zeros((sc.nbdry, 64 + 2 * G))
    for p, b in enumerate(d0.boxes):
        Ug[:, b[1] + G:b[3] + G + 1, b[0] + G:b[2] + G + 1] = d0.U[p][:, G:-G, G:-G]
        if d0.B[p] is not None:
            Bg[:, b[0] + G:b[2] + G + 1] = d0.B[p][:, G:-G]
    wf, wb = O.station_values((0, 0, 63, 31), sc.dx, Ug, Bg, fx, [(3.21, 0.45)])
    np.testing.assert_array_equal(rc["fault"][0, 0], wf[0])
    np.testing.assert_array_equal(rc["body"][0, 0], wb[0])
    for s in sts:
        s.close()
    h.close()
    for lv in lvs:
        lv.close()
    ctx.close()


def test_station_files_in_the_reference_format(cuda_lib, tmp_path):
    from tetemoko_gb300.stations import Stations, read_station_file
    sc, ctx, lvl, Ug, Bg = _setup(A.TMK_PREC_FP64)
    st = Stations(lvl, [1.234], [(0.95, 0.55)], capacity=8)
    st.attach()
    for k in range(3):
        lvl.step(k * sc.dt(), sc.dt())
    rec = st.read()
    prefix = str(tmp_path / "run_")
    st.write_files(prefix, 0, rec, create=True)
    fnames, bnames = st.file_names(prefix, 0)
    assert os.path.basename(fnames[0]) == "run_Fx1.2340z0.0000.L0.dat"
    assert os.path.basename(bnames[0]) == "run_Bx0.9500y0.5500z0.0000.L0.dat"
    with open(fnames[0], "rb") as fh:
        head = fh.read(200).split(b"\n")
    assert head[0] == b"#number of values = 11" and head[1] == b"#size of real = 8"
    assert head[2].startswith(b"#time\tVx\tVz\tV\tsxy") and head[2].endswith(b"\tlevel\tprocID")
    cols, r = read_station_file(fnames[0])
    assert r.shape == (3, 14) and cols[-2:] == ["level", "procID"]
    np.testing.assert_array_equal(r[:, 0], rec["time"])
    np.testing.assert_array_equal(r[:, 1:12], rec["fault"][:, 0])
    cols, r = read_station_file(bnames[0])
    assert r.shape == (3, 25) and cols[1] == "v_x^1"
    np.testing.assert_array_equal(r[:, 1:23], rec["body"][:, 0])
    st.close()
    lvl.close()
    ctx.close()


@pytest.mark.parametrize("which", ["fault_only", "body_only"])
def test_stations_of_one_kind_only(cuda_lib, which):
    """A station set with fault stations alone (or body stations alone) reads
    back records of the right shapes."""
    from tetemoko_gb300.stations import Stations
    sc, ctx, lvl, Ug, Bg = _setup(A.TMK_PREC_FP64)
    fx, bxy = (FAULT_X, []) if which == "fault_only" else ([], BODY_XY[:2])
    st = Stations(lvl, fx, bxy, capacity=8)
    st.attach()
    for k in range(3):
        lvl.step(k * sc.dt(), sc.dt())
    rec = st.read()
    assert rec["time"].shape == (3,)
    assert rec["fault"].shape == (3, len(fx), sc.nbdry)
    assert rec["body"].shape == (3, len(bxy), 22)
    st.close()
    lvl.close()
    ctx.close()
