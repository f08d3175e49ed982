"""The oracle's RANS-SA restatement is pinned to the reference's own outputs.

The fixtures rans_naca_og64 and rans_channel_tri were produced by the
reference's RANSTurbulenceSASolver compiled in place
(tests/golden/make_golden.py).  The restatement (oracle/fv_oracle.cpp,
struct Rans) must reproduce the wall distance, the mean-flow field and
nu-tilde bit for bit, and the five residual norms to the last few ulps (the
L2 sums are OpenMP reductions whose order depends on the thread count).
The fixtures were written on an x86-64 host; std::hypot and std::pow may
differ in the last bit on another host's maths library, so off x86-64 the
comparison is within 1e-10 relative.
"""
import platform

import numpy as np
import pytest

from helpers import GAMMA, case_of, load_golden, poly_of, rel_err
from oracle import port

FLUX = {"rusanov": 0, "hllc": 1}
GRAD = {"lsq": 0, "gg": 1}
X86 = platform.machine() in ("x86_64", "AMD64")


def _bcs(specs, names):
    out = [{"type": "noslip"} for _ in names]
    for spec in specs:
        p = spec.split(":")
        i = names.index(p[0])
        if p[1] == "noslip":
            b = {"type": "noslip", "wall_u": float(p[2]) if len(p) > 2 else 0.0,
                 "wall_v": float(p[3]) if len(p) > 3 else 0.0}
            if len(p) > 4:
                b["wall_T"] = float(p[4])
        elif p[1] == "outflow":
            b = {"type": "outflow"}
        else:
            r, u, v, pr = map(float, p[2:6])
            b = {"type": "farfield", "state": (r, r * u, r * v, pr / (GAMMA - 1.0) + 0.5 * r * (u * u + v * v)),
                 "nut": float(p[6]) if len(p) > 6 else 0.0}
        out[i] = b
    return out


def _ic(spec):
    r, u, v, p = map(float, spec.split(":")[1:5])
    return {"mode": "free", "rho": r, "u": u, "v": v, "p": p}


CASES = [("rans_naca_og64", "rusanov", "lsq"), ("rans_naca_og64", "hllc", "gg"),
         ("rans_channel_tri", "rusanov", "lsq"), ("rans_channel_tri", "rusanov", "gg")]


@pytest.mark.parametrize("name,flux,grad", CASES)
def test_oracle_rans_matches_reference(name, flux, grad):
    g = load_golden(name)
    case = case_of(g)
    poly = poly_of(g)
    om = port.OracleMesh(poly)
    r = port.OracleRANS(om, _bcs(case["bc"], poly.patch_names), GAMMA, case["R"], case["mu"], case["Pr"], case["Prt"],
                        case["cfl"], _ic(case["ic"]), case["nut0"], flux=FLUX[flux], gradient=GRAD[grad])
    hist = r.run(case["steps"])
    field, nut, walld = r.get()
    tag = f"{flux}_{grad}"
    assert np.array_equal(walld, g["walld"])
    if X86:
        assert np.array_equal(field, g[f"field_{tag}"])
        assert np.array_equal(nut, g[f"nut_{tag}"])
        np.testing.assert_allclose(hist, g[f"hist_{tag}"], rtol=1e-12, atol=0)
    else:
        assert rel_err(field, g[f"field_{tag}"]) <= 1e-10
        assert rel_err(nut, g[f"nut_{tag}"]) <= 1e-10
        np.testing.assert_allclose(hist, g[f"hist_{tag}"], rtol=1e-10, atol=0)
