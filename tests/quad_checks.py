"""Checks shared by the quad generator tests."""
import numpy as np


def tri_key(t):
    t = [int(v) for v in t]
    k = t.index(min(t))
    return tuple(t[k:] + t[:k])  # rotation-normalised, winding kept


def check_quadization(tris, quads, num_degenerate):
    """Every input tri appears exactly once: a quad (a, b, c, d) holds the tris (a, b, c) and
    (a, c, d) (the two tris of quad setup), a degenerate quad (a, b, c, c) one tri; the pairs of a
    quad share the edge (a, c); tris keep their input order by first tri."""
    want = sorted(tri_key(t) for t in tris)
    got = []
    deg = 0
    for q in np.asarray(quads, np.int64):
        a, b, c, d = (int(v) for v in q)
        if c == d:
            got.append(tri_key((a, b, c)))
            deg += 1
        else:
            got.append(tri_key((a, b, c)))
            got.append(tri_key((a, c, d)))
    assert deg == num_degenerate
    assert sorted(got) == want
    assert len(quads) == len(tris) - (len(tris) - deg) // 2
