"""The iterate driver flow (osb.drv.f90) on reference-format files: parameter
file -> H0/RES/DEP -> preconditioner build (saved with sVOSB > 0, reloaded with
sVOSB < 0) -> PIST with the PT basis file (sPT != 0)."""
import numpy as np
import pytest

from scalit_gb300 import capi, hamiltonian as hm, osb, refio

pytestmark = pytest.mark.gpu


def test_driver_end_to_end(lib, tmp_path):
    p = hm.workload("tri-24x32x20")
    e0 = float(p.RES.min())
    inp = refio.OSBInput(sBJ=(20, 1e-4), sQMR=(500, 1e-4), sConv=(e0, 1e-11, 0, 5, 400, 20, 1),
                         sOSBW=(e0, 0.0, 0.0, 0), sVOSB=1, sPT=1,
                         VOSBFile=str(tmp_path / "VOSB.dat"), EigFile=str(tmp_path / "EIG.dat"),
                         PTFile=str(tmp_path / "PT.dat"))
    inp = refio.write_problem_files(p, tmp_path, inp)
    text = (tmp_path / "input.txt").read_text()
    lines = []
    o = osb.OSB.read(text)
    assert o.load_init_data()
    o.prog_diag(log=lines.append)
    st, eig, res, info = o.prog_pist_eig(log=lines.append)
    x = np.random.default_rng(0).standard_normal(p.N)
    z_built = o.ctx.px(x)
    o.close()
    assert st > 0
    assert any("Jacobi Effi" in s for s in lines) and any("Eigen Values" in s for s in lines)
    cnt, ritz, hmat, vj = refio.load_pist_basis(inp.PTFile)
    assert cnt == st
    np.testing.assert_allclose(np.linalg.eigvalsh(hmat), np.sort(ritz), atol=1e-12)
    assert np.abs(vj.T @ vj - np.eye(cnt)).max() < 1e-10
    # reload the saved preconditioner (sVOSB < 0): same P*X
    text2 = text.replace("0 1 0 0 1", "0 -1 0 0 0")
    inp2 = refio.read_input(text2)
    assert inp2.sVOSB == -1 and inp2.VOSBFile == inp.VOSBFile
    o2 = osb.OSB(inp2)
    o2.load_init_data()
    o2.prog_diag(log=None)
    np.testing.assert_array_equal(o2.ctx.px(x), z_built)
    o2.close()
