"""The device-resident ik loop (clowns_session_*) against the oracle running the
same loop (1sub-momentum.F90:41-60): same number of ik passes, pressure and
face velocities within 1e-8 relative (each pass carries a solve at 1e-10)."""
import numpy as np
import pytest

from cases import small_cases

pytestmark = pytest.mark.gpu


def _oracle_loop(ora, case, d0, eps0):
    cls = ora.set_nflag(case)
    sm = ora.init_matrix(case, cls)
    c = case.copy()
    c.f = cls.f.copy()
    p = np.zeros(case.inne2 + 2)
    un = case.un.copy()
    ik = 0
    while True:
        c.un = un
        sy = ora.rows_rhs_assemble(c, cls, sm)
        if sy.dmax < d0:
            break
        ik += 1
        if ik > 1000:
            break
        r = ora.pcgpme(sy.alu, sy.llu, sy.de[1:], sy.b[1:], sy.mnoe, eps=eps0)
        p, un = ora.correct(c, cls, sy, r.x, p, un)
    return ik, sy.dmax, p, un, cls


@pytest.mark.parametrize("idx", [1, 2])
def test_session_ik_loop_matches_oracle(gpu, ora, idx):
    label, case = small_cases()[idx]
    d0, eps0 = 1e-5, 1e-12
    ik_o, dmax_o, p_o, un_o, cls = _oracle_loop(ora, case, d0, eps0)
    s = gpu.Session(case)
    s.set_fields(case.nf, case.nfb, case.f, case.fb, case.a, case.un, case.sp, np.zeros(case.inne2 + 2))
    ifln, isfn = s.classify()
    assert ifln == cls.ifln and isfn == cls.isfn
    out = s.pressure_loop(case.dt, d0=d0, eps0=eps0)
    got = s.fields()
    s.close()
    assert out["icon"] == 0
    assert out["ik"] == ik_o >= 1
    assert np.array_equal(got["nf"], cls.nf) and np.array_equal(got["nfb"], cls.nfb)
    assert np.linalg.norm(got["p"] - p_o) <= 1e-8 * np.linalg.norm(p_o)
    assert np.linalg.norm(got["un"] - un_o) <= 1e-8 * np.linalg.norm(un_o)
    assert out["dmax"] < d0 and dmax_o < d0
