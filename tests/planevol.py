"""Exact liquid fraction of a box cut by a plane, independent of the reference's tet clip.

Liquid is the side n.x < c (negative signed distance, as in src/VF.jl:251).  With
x = x0 + s*a (s in [0,1]^3) the fraction is vol{s : m.s < alpha}, m_i = n_i a_i, and
negative m_i are folded by s_i -> 1 - s_i.  For positive m the inclusion-exclusion form
F = sum_v (-1)^|v| max(0, alpha - m.v)^3 / (6 m1 m2 m3) is evaluated in 60-digit mpmath,
so cancellation does not matter.  Components with |m_i| tiny are handled by the 2D/1D
forms of the same sum.
"""
import itertools

import mpmath

mpmath.mp.dps = 60


def box_fraction(n, c, lo, hi):
    m = []
    alpha = mpmath.mpf(c)
    for d in range(3):
        a = mpmath.mpf(hi[d]) - mpmath.mpf(lo[d])
        nd = mpmath.mpf(n[d])
        alpha -= nd * mpmath.mpf(lo[d])
        md = nd * a
        if md < 0:
            alpha -= md
            md = -md
        m.append(md)
    act = [x for x in m if x != 0]
    k = len(act)
    if k == 0:
        return 1.0 if alpha > 0 else 0.0
    tot = mpmath.mpf(0)
    for v in itertools.product((0, 1), repeat=k):
        t = alpha - sum(mi * vi for mi, vi in zip(act, v))
        if t > 0:
            tot += (-1) ** sum(v) * t ** k
    den = mpmath.factorial(k)
    for mi in act:
        den *= mi
    return float(tot / den)
