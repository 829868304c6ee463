"""The oracle restatement (FAITHFUL32 mode) against golden vectors produced
by the reference's own compute shaders (tests/golden/make_golden.py): bit
for bit, particles after every step and the grid after the last one."""
import numpy as np
import pytest

from oracle import oracle as O
from tests._util import golden_names, load_golden


@pytest.mark.parametrize("name", golden_names())
@pytest.mark.parametrize("threads", [1, 4])
def test_faithful32_matches_reference_bitwise(name, threads):
    s, z = load_golden(name)
    o = O.OracleSim(s, mode=O.FAITHFUL32, threads=threads).upload_std140(z["pxm0"], z["pv0"], *s.std140()[2:])
    o.init()
    _, pv, _, _ = o.state_std140()
    assert np.array_equal(pv, z["pv_init"]), "density after init differs"
    steps = int(z["steps"])
    for k in range(1, steps + 1):
        o.step()
        pxm, pv, fe, fp = o.state_std140()
        assert np.array_equal(pxm.view(np.int32), z[f"pxm_{k}"].view(np.int32)), f"pxm step {k}"
        assert np.array_equal(pv, z[f"pv_{k}"]), f"pv step {k}"
        fe9 = fe.reshape(-1, 4, 4)[:, :3, :3].reshape(-1, 9)
        fp9 = fp.reshape(-1, 4, 4)[:, :3, :3].reshape(-1, 9)
        assert np.array_equal(fe9.view(np.int32), z[f"fe_{k}"].view(np.int32)), f"FE step {k}"
        assert np.array_equal(fp9.view(np.int32), z[f"fp_{k}"].view(np.int32)), f"FP step {k}"
    gv, gf = o.grid_fixed()
    nodes = z["grid_nodes"]
    nz = np.nonzero((gv != 0).any(1) | (gf != 0).any(1))[0]
    assert np.array_equal(nz, nodes)
    assert np.array_equal(gv[nodes], z["grid_gv"])
    assert np.array_equal(gf[nodes, :3], z["grid_gf"][:, :3])
    vstar = o.grid()["vstar"]
    assert np.array_equal(vstar[nodes].astype(np.float32).view(np.int32),
                          z["grid_gvn"][:, :3].astype(np.float32).view(np.int32))
    assert np.array_equal(o.colliders().astype(np.float32), z["colliders_cx"][:, :3])


def test_reference_compiled_matches_port_when_available():
    """Where the reference tree (or its translated shaders) is present, run
    both on a fresh random scene, not only on the committed fixtures."""
    if O.ref_lib() is None:
        pytest.skip("compiled reference shaders unavailable")
    from snow_gb300 import scenes
    s = scenes.small_scene(n=1200, grid_edge=24, seed=99, v0=(0.7, -3.0, 0.2))
    bufs = s.std140()
    r = O.RefSim(s, threads=4).upload_std140(*bufs).init()
    o = O.OracleSim(s, mode=O.FAITHFUL32, threads=4).upload_std140(*bufs).init()
    for _ in range(2):
        r.update()
        o.step()
    for a, b in zip(r.state_std140(), o.state_std140()):
        assert np.array_equal(a.view(np.int32), b.view(np.int32))
