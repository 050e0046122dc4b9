"""Generates tests/golden/kat.npz: analytic known-answer cases for the raster path.

The reference has no tests and cannot run here, so these cases are derived from the
reference's documented conventions instead of from its outputs:

* coverage is point sampling at pixel centres (x+0.5, y+0.5) (the scan records of
  quad_setup.glsl:334-339 start at (-0.5, 0.5) and raster.glsl:116-140 rounds the edge
  crossings accordingly); pixels whose centre lies exactly on an edge are excluded from the
  comparison since either side may own them;
* colours are perspective-correct barycentric interpolations of the vertex colours
  (shading.glsl:116-165), here computed by intersecting the pixel ray with the triangle's
  plane in float64;
* blending is front to back, out += c*a*T, T *= 1-a, then out += T*background
  (shading.glsl:279-280, 312).

Each case stores screen-space vertices (x, y, view depth), RGBA8 vertex colours, the
viewport and background, and the expected per-pixel coverage mask and colour. Run from the
repository root: ``python tests/golden/make_golden.py``.
"""
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
FOV_Y = math.radians(60.0)


def unproject(sx, sy, d, w, h):
    ty = math.tan(float(np.float32(FOV_Y)) * 0.5)
    tx = ty * (w / h)
    return np.array([(2 * sx / w - 1) * tx * d, (2 * sy / h - 1) * ty * d, -d])


def ray(px, py, w, h):
    ty = math.tan(float(np.float32(FOV_Y)) * 0.5)
    tx = ty * (w / h)
    return np.array([(2 * (px + 0.5) / w - 1) * tx, (2 * (py + 0.5) / h - 1) * ty, -1.0])


def edge_side(p, a, b):
    return (b[0] - a[0]) * (p[1] - a[1]) - (b[1] - a[1]) * (p[0] - a[0])


def rasterize_case(tris, colors, w, h, bg):
    """tris: list of 3x3 (sx, sy, depth); colors: list of 3 RGBA8 tuples per tri."""
    covered = np.zeros((len(tris), h, w), bool)
    on_edge = np.zeros((h, w), bool)
    frag = {}
    for t, tri in enumerate(tris):
        s = [np.array(v[:2], float) for v in tri]
        area = edge_side(s[2], s[0], s[1])
        for y in range(h):
            for x in range(w):
                pc = np.array([x + 0.5, y + 0.5])
                e = [edge_side(pc, s[i], s[(i + 1) % 3]) * np.sign(area) for i in range(3)]
                if min(e) > 0:
                    covered[t, y, x] = True
                elif min(e) == 0 and max(e) >= 0:
                    on_edge[y, x] = True
        P = [unproject(v[0], v[1], v[2], w, h) for v in tri]
        n = np.cross(P[1] - P[0], P[2] - P[0])
        for y, x in zip(*np.nonzero(covered[t])):
            d = ray(x, y, w, h)
            tt = np.dot(n, P[0]) / np.dot(n, d)
            X = d * tt
            # barycentrics of X in the 3D triangle
            a_tot = np.dot(n, n)
            b1 = np.dot(np.cross(P[2] - P[1], X - P[1]), n) / a_tot
            b2 = np.dot(np.cross(P[0] - P[2], X - P[2]), n) / a_tot
            b3 = 1.0 - b1 - b2
            c = np.array(colors[t], float) / 255.0
            col = b1 * c[0] + b2 * c[1] + b3 * c[2]
            frag.setdefault((y, x), []).append((tt, t, col))
    image = np.zeros((h, w, 4))
    counts = np.zeros((h, w), np.int32)
    for y in range(h):
        for x in range(w):
            fr = sorted(frag.get((y, x), []), key=lambda f: (f[0], f[1]))  # nearest first
            counts[y, x] = len(fr)
            out, T = np.zeros(3), 1.0
            for _, _, col in fr:
                out += col[:3] * col[3] * T
                T *= 1.0 - col[3]
            image[y, x, :3] = np.clip(out + T * np.array(bg[:3]), 0, 1)
            image[y, x, 3] = 1.0
    return covered, on_edge, image, counts


CASES = {
    # one right triangle at constant depth
    "right_triangle": dict(w=64, h=64, bg=(0.0, 0.0, 1.0, 1.0),
                           tris=[[(8, 8, 10.0), (40, 8, 10.0), (8, 40, 10.0)]],
                           colors=[[(255, 0, 0, 128)] * 3]),
    # two overlapping triangles, near one listed second
    "two_layers": dict(w=64, h=48, bg=(0.2, 0.2, 0.2, 1.0),
                       tris=[[(4, 4, 20.0), (60, 6, 20.0), (30, 44, 20.0)],
                             [(10, 40, 5.0), (50, 42, 5.0), (32, 2, 5.0)]],
                       colors=[[(0, 255, 0, 200)] * 3, [(255, 0, 255, 100)] * 3]),
    # perspective-correct interpolation: slanted triangle with distinct vertex colours
    "slanted_gradient": dict(w=96, h=64, bg=(0.0, 0.0, 0.0, 1.0),
                             tris=[[(6, 5, 2.0), (90, 12, 40.0), (40, 60, 9.0)]],
                             colors=[[(255, 0, 0, 255), (0, 255, 0, 255), (0, 0, 255, 255)]]),
    # three mutually intersecting slanted triangles (per-pixel order changes across the image)
    # (no exactly horizontal edges: the reference's scan record of such an edge is NaN, so
    # its constraint drops out and only the 8-row y-range bounds the triangle)
    "intersecting": dict(w=80, h=80, bg=(1.0, 1.0, 1.0, 1.0),
                         tris=[[(5, 10, 2.0), (75, 11.3, 30.0), (40, 70, 15.0)],
                               [(5, 70, 30.0), (75, 68.6, 2.0), (40, 5, 15.0)],
                               [(10, 40, 15.0), (70, 20, 15.0), (60, 75, 15.0)]],
                         colors=[[(255, 0, 0, 150)] * 3, [(0, 255, 0, 150)] * 3,
                                 [(0, 0, 255, 150)] * 3]),
}


def main():
    out = {}
    for name, c in CASES.items():
        covered, on_edge, image, counts = rasterize_case(c["tris"], c["colors"], c["w"], c["h"], c["bg"])
        out[f"{name}/tris"] = np.array(c["tris"], np.float64)
        out[f"{name}/colors"] = np.array(c["colors"], np.uint8)
        out[f"{name}/size"] = np.array([c["w"], c["h"]], np.int32)
        out[f"{name}/bg"] = np.array(c["bg"], np.float32)
        out[f"{name}/covered"] = covered
        out[f"{name}/on_edge"] = on_edge
        out[f"{name}/image"] = image.astype(np.float32)
        out[f"{name}/counts"] = counts
    np.savez_compressed(os.path.join(HERE, "kat.npz"), **out)
    print("wrote", os.path.join(HERE, "kat.npz"), "cases:", ", ".join(CASES))


if __name__ == "__main__":
    main()
