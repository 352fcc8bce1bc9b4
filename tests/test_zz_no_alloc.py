"""rfgpu_residual_noalloc: the residual entry point that allocates no device
memory, for callers that may not allocate (a host whose device memory is
budgeted once at start-up, or code running where the CUDA runtime must not
be asked for memory).  Its face-flux and residual scratch is the library's
fixed static device array.  Checked through the C ABI against rfgpu_residual
on two calls in a row (the array keeps the previous call's contents), and the
size limit is reported as RFGPU_ERR_NOALLOC_LIMIT.  Kept in a file of its own
that pytest collects last."""
import numpy as np
import pytest

from rocflupicl_gb300 import case as K
from rocflupicl_gb300 import engine as E

pytestmark = pytest.mark.gpu


def _cases():
    yield K.shock_tube(24, numerics=K.Numerics(venkatGuard=1))
    yield K.tet_shock_box(4, seed=5, numerics=K.Numerics(spaceDiscr=K.DISCR_UPW_ROE,
                                                         venkatGuard=1))
    yield K.mixed_box(6, numerics=K.Numerics(spaceDiscr=K.DISCR_UPW_HLLC, venkatGuard=1))


@pytest.mark.parametrize("prec", [K.PREC_FP64, K.PREC_MIXED, K.PREC_SPLIT])
def test_noalloc_residual_matches_residual_twice(prec):
    for c in _cases():
        r = E.Region(c, precision=prec)
        ref = r.residual()
        scale = np.abs(ref).max()
        for _ in range(2):                       # two calls in a row
            got = r.residual_noalloc()
            # both paths bit-identical: the scratch kernels repeat the region
            # kernels' arithmetic (the mixed path's compensated FP32 sums too)
            assert np.array_equal(got, ref), np.abs(got - ref).max() / scale
        r.close()


def test_noalloc_after_other_region_and_limit():
    # a second, different region reuses the same static scratch
    a = E.Region(K.tet_shock_box(3, seed=1, numerics=K.Numerics(venkatGuard=1)))
    b = E.Region(K.shock_tube(40, numerics=K.Numerics(venkatGuard=1)))
    ra, rb = a.residual(), b.residual()
    assert np.array_equal(a.residual_noalloc(), ra)
    assert np.array_equal(b.residual_noalloc(), rb)
    assert np.array_equal(a.residual_noalloc(), ra)
    a.close()
    b.close()
    # 40^3 x 6 tets need ~60 MB of FP64 scratch, more than the fixed 32 MiB
    big = E.Region(K.tet_shock_box(40, seed=2, numerics=K.Numerics(venkatGuard=1)))
    with pytest.raises(E.EngineError) as ei:
        big.residual_noalloc()
    assert ei.value.code == E.ERR_NOALLOC_LIMIT
    big.close()
