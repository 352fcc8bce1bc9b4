"""A case read from the reference's grid and flow files runs through the
engine exactly as the case it was written from: the binary grid keeps the
coordinates bit for bit, so mesh, residual and a few steps agree bitwise; the
state written back as a flow file reads back unchanged."""
import numpy as np
import pytest

from rocflupicl_gb300 import case as K
from rocflupicl_gb300 import engine as E
from rocflupicl_gb300 import rfluio as IO

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [K.PREC_FP64, K.PREC_MIXED])
def test_case_from_files_matches_source(tmp_path, prec):
    num = K.Numerics(spaceDiscr=K.DISCR_UPW_ROE, precision=prec, venkatGuard=1)
    c = K.tet_shock_box(5, seed=12, numerics=num)
    gp, fp = str(tmp_path / "box.grd"), str(tmp_path / "box.flo")
    IO.write_grid_binary(gp, IO.grid_of_mesh(c.mesh))
    K.write_flow(fp, c.cv, binary=True)
    f = K.from_files(gp, fp, c.bcs, num, binary=True)
    a, b = E.Region(c), E.Region(f)
    assert np.array_equal(a.residual(), b.residual())
    a.solve(n_steps=3)
    b.solve(n_steps=3)
    cva, _ = a.download()
    cvb, _ = b.download()
    assert np.array_equal(cva, cvb)
    out = str(tmp_path / "out.flo")
    K.write_flow(out, cvb, time=b.time()[0], binary=True)
    assert np.array_equal(IO.read_flow_binary(out).cv, cvb)
    a.close()
    b.close()
