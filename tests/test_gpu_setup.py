"""Setup on the device: the physical cells' geometry (volumes, centroids,
face areas and centres) and wall distance computed by kernels equal the
host setup's bit for bit, on a curvilinear C-grid airfoil with a wake cut
(the reference's rae2822 case, where present), a stretched SST flat plate,
a skewed two-block case and a bump channel; and the solver runs from the
device-built setup exactly as from the host one."""
import numpy as np
import pytest

from refcases_common import case_input, have_case

pytestmark = pytest.mark.gpu


def _inputs(tmp):
    from aither_gb300 import cases
    out = [cases.sst_plate(str(tmp / "sst"), ni=64, nj=48, nk=3, name="sst")[0],
           cases.block_pair(str(tmp / "pair"), orient=5, physics="sst", name="pair")[0],
           cases.bump_channel(str(tmp / "bump"), 24, 12, 6, 0.08, 0.6, name="bump")[0]]
    if have_case("rae2822"):
        out.append(case_input("rae2822"))
    return out


def test_device_geometry_and_wall_distance_equal_host(tmp_path):
    from aither_gb300 import Setup
    for inp in _inputs(tmp_path):
        h = Setup(inp)
        d = Setup(inp, device=0)
        for b in range(h.counts()[1]):
            gh, gd = h.geometry(b), d.geometry(b)
            for key in ("vol", "center", "width", "fareai", "fareaj", "fareak"):
                assert np.array_equal(gh[key], gd[key]), (inp, b, key)
            vh, vd = h.block_view(b), d.block_view(b)
            n = vh.ncell_padded
            wh = np.ctypeslib.as_array(vh.wall_dist, shape=(n,))
            wd = np.ctypeslib.as_array(vd.wall_dist, shape=(n,))
            assert np.array_equal(wh, wd), (inp, b)


def test_solver_from_device_setup_equals_host_setup(tmp_path):
    from aither_gb300 import Batch, Context, Setup
    ctx = Context(0)
    inp = _inputs(tmp_path)[0]
    res = []
    for dev in (None, 0):
        b = Batch(ctx, Setup(inp, device=dev))
        b.iterate(5)
        res.append(b.field(0, "STATE"))
        b.close()
    assert np.array_equal(res[0], res[1])
    ctx.close()
