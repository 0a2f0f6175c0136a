"""Generate the known-answer fixtures of tests/golden/ (run from the repo root).

The reference ships no tests or golden vectors and cannot be compiled here
(Fortran + MPI, no Fortran compiler), so the fixtures come from mathematics:

kat_stencils.json   exact rational values (sympy) of the reference's 7-point
                    stencils (deriv.f90:12-25) applied to monomials x^n on an
                    offset grid, the exact derivative they must reproduce, and
                    the Fourier symbols of D2/D1 at a few phases.
kat_rk3.json        the stability polynomial of the 2N-storage RK3 of
                    run.f90:46-54 (A = 0, -2/3, -1; B = 1/3, 1, 1/2), derived
                    symbolically, and its values at a few complex z.
oracle_regress.json a 12^3 FP64 real-time run of the CPU oracle from a seeded
                    state (checksums of psi after 10 steps); it freezes the
                    oracle so a later change to it cannot go unnoticed.
"""
import json
import os
import sys

import sympy as sp

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def stencils():
    h, x0 = sp.Rational(1, 2), sp.Rational(3, 4)
    d2w = [2, -27, 270, -490, 270, -27, 2]
    d1w = [-1, 9, -45, 0, 45, -9, 1]
    out = {"h": str(h), "x0": str(x0), "d2": [], "d1": []}
    x = sp.Symbol("x")
    for n in range(0, 10):
        f = x ** n
        vals = [f.subs(x, x0 + m * h) for m in range(-3, 4)]
        d2 = sum(w * v for w, v in zip(d2w, vals)) / (180 * h ** 2)
        d1 = sum(w * v for w, v in zip(d1w, vals)) / (60 * h)
        out["d2"].append({"n": n, "stencil": str(sp.nsimplify(d2)), "exact": str(sp.diff(f, x, 2).subs(x, x0))})
        out["d1"].append({"n": n, "stencil": str(sp.nsimplify(d1)), "exact": str(sp.diff(f, x).subs(x, x0))})
    th = sp.Symbol("theta")
    sym2 = (sum(w * sp.cos((m - 3) * th) for m, w in enumerate(d2w)) / 180)
    out["d2_symbol_at"] = {str(v): float(sym2.subs(th, v)) for v in (sp.pi / 4, sp.pi / 2, sp.pi)}
    return out


def rk3():
    z = sp.Symbol("z")
    A = [0, sp.Rational(-2, 3), -1]
    B = [sp.Rational(1, 3), 1, sp.Rational(1, 2)]
    psi, w = sp.Integer(1), sp.Integer(0)
    for a, b in zip(A, B):
        w = a * w + z * psi
        psi = psi + b * w
    poly = sp.expand(psi)
    coeffs = [str(poly.coeff(z, k)) for k in range(5)]
    pts = [complex(0, 0.3), complex(-0.5, 0.2), complex(0, 1.5), complex(-2.0, 0)]
    vals = [[p.real, p.imag, complex(poly.subs(z, sp.nsimplify(p.real) + sp.I * sp.nsimplify(p.imag))).real,
             complex(poly.subs(z, sp.nsimplify(p.real) + sp.I * sp.nsimplify(p.imag))).imag] for p in pts]
    return {"coeffs": coeffs, "values": vals}


def oracle_regress():
    import numpy as np
    from oracle.pyoracle import Oracle
    from tests.helpers import params, smooth_state
    p = params(n=(12, 12, 12), L=(6.0, 6.0, 6.0), pot="harmonic", harm=(2.0, 3.0, 4.0), omega=0.3, dt=0.01)
    o = Oracle(p)
    o.set_psi(smooth_state(p, seed=7))
    o.step_rt(10)
    a = o.get_psi()
    d = o.diag()
    return {"n": 12, "L": 6.0, "harm": [2.0, 3.0, 4.0], "omega": 0.3, "dt": 0.01, "steps": 10, "seed": 7,
            "sum_re": float(a.real.sum()), "sum_im": float(a.imag.sum()),
            "sum_abs2": float((np.abs(a) ** 2).sum()), "psi_000": [float(a[0, 0, 0].real), float(a[0, 0, 0].imag)],
            "psi_mid": [float(a[6, 5, 4].real), float(a[6, 5, 4].imag)], "energy": d["energy"], "mu": d["mu"]}


if __name__ == "__main__":
    with open(os.path.join(HERE, "kat_stencils.json"), "w") as f:
        json.dump(stencils(), f, indent=1)
    with open(os.path.join(HERE, "kat_rk3.json"), "w") as f:
        json.dump(rk3(), f, indent=1)
    with open(os.path.join(HERE, "oracle_regress.json"), "w") as f:
        json.dump(oracle_regress(), f, indent=1)
    print("written")
