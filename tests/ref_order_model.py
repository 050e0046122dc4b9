"""Independent model of the reference-order mode, written from the reference GLSL in float32
Python scalars, used to check the oracle's C++ restatement on small scenes.

raster_low.glsl / raster_high.glsl (block and half-block lists, keys, promotion, errors),
raster.glsl:142-176 (centroids, block keys), shading.glsl:107-314 (lit RGBA8 samples, 3-deep
window), raster.glsl:361-398 (segment saturation). Ties of equal keys and blocks of <= 3 tris are
in primitive-id order (the reference's arrival order is not deterministic).
"""
from __future__ import annotations

import math

import numpy as np

F = np.float32
INF = F(np.inf)


def bitsf(u):
    return np.array([u], np.uint32).view(np.float32)[0]


def fbits(f):
    return int(np.array([f], np.float32).view(np.uint32)[0])


def f2i(x):
    x = F(x)
    if x != x:
        return 0
    if x >= F(2147483647.0):
        return 2147483647
    if x <= F(-2147483648.0):
        return -2147483648
    return int(np.trunc(x))


def f2u(x):
    x = F(x)
    if x != x or x <= 0:
        return 0
    if x >= F(4294967295.0):
        return 4294967295
    return int(np.trunc(x))


def fmax(a, b):
    a, b = F(a), F(b)
    if a != a:
        return b
    if b != b:
        return a
    return max(a, b)


def fmin(a, b):
    a, b = F(a), F(b)
    if a != a:
        return b
    if b != b:
        return a
    return min(a, b)


def sat(v):
    return fmin(fmax(v, F(0)), F(1))


def pow_series(x, y):
    """x^y by exp2(y log2 x): the atanh series for log2 and a Taylor series for 2^f."""
    x, y = F(x), F(y)
    if x != x:
        return x
    if x <= 0:
        return F(0) if x == 0 else F(np.nan)
    if x == INF:
        return INF if y > 0 else F(0)
    e = 0
    b = fbits(x)
    if (b >> 23) & 0xFF == 0:
        x = x * F(8388608.0)
        b = fbits(x)
        e = -23
    e += ((b >> 23) & 0xFF) - 127
    m = bitsf((b & 0x7FFFFF) | 0x3F800000)
    if m > F(math.sqrt(2.0)):
        m = m * F(0.5)
        e += 1
    t = (m - F(1)) / (m + F(1))
    t2 = t * t
    s = F(1) / F(13)
    for c in (11, 9, 7, 5, 3):
        s = s * t2 + F(1) / F(c)
    s = s * t2 + F(1)
    ln_m = (F(2) * t) * s
    l2 = F(e) + ln_m * F(1.0 / math.log(2.0))
    z = y * l2
    if z >= F(128):
        return INF
    if z < F(-149):
        return F(0)
    k = F(np.floor(z))
    u = (z - k) * F(math.log(2.0))
    p = F(1) / F(3628800)
    for fct in (362880, 40320, 5040, 720, 120, 24, 6):
        p = p * u + F(1) / F(fct)
    p = p * u + F(0.5)
    p = p * u + F(1)
    p = p * u + F(1)
    ki = int(k)
    if ki < -126:
        p = p * bitsf((ki + 126 + 127) << 23)
        ki = -126
    return p * bitsf((ki + 127) << 23)


def decode_rgba8(c):
    s = F(1) / F(255)
    return [F(float((c >> (8 * i)) & 0xFF)) * s for i in range(4)]


class Model:
    def __init__(self, scene, out, flags=0):
        self.sc = scene
        self.o = out
        self.flags = flags
        self.w, self.h = scene.width, scene.height
        self.bcx = (self.w + 31) // 32
        self.scan = out["tri_scan"]
        self.depth = out["tri_depth"]
        self.bary = out["tri_bary"]
        self.verts = out["quad_verts"]
        self.src = out["quad_source"]
        self.normals = out["tri_normals"]
        cfg = scene.config
        self.bg = [F(cfg.background_color[i]) for i in range(3)]
        self.sun_dir = [F(cfg.sun_dir[i]) for i in range(3)]
        self.sun_color = [F(cfg.sun_color[i]) for i in range(3)]
        self.amb_color = [F(cfg.ambient_color[i]) for i in range(3)]
        self.sun_power, self.amb_power = F(cfg.sun_power), F(cfg.ambient_power)

    # ---- coverage (generateRowTris with a row-group start; rasterBinStep)
    def rows(self, tri, bin_x, bin_y, group):
        sc = self.scan[tri]
        rows = [(31, 0)] * 32
        shift = 3 if group == 8 else 2
        ymin, ymax = int(sc[3] & 0xFFFF) - bin_y, int(sc[3] >> 16) - bin_y
        ming = min(max(ymin, 0), 31) >> shift
        maxg = min(max(ymax, 0), 31) >> shift
        sx, sy = F(bin_x), F(bin_y + ming * group)
        mn, mx, st = [], [], []
        for i in range(3):
            step = bitsf(sc[4 + i])
            v = bitsf(sc[i]) + (step * sy - sx)
            xneg = (int(sc[7]) >> i) & 1
            mn.append(-INF if xneg else v)
            mx.append(v if xneg else INF)
            st.append(step)
        for r in range(ming * group, maxg * group + group):
            fl = fmax(fmax(mn[0], mn[1]), fmax(mn[2], F(0)))
            fh = fmin(fmin(mx[0], mx[1]), fmin(mx[2], F(32)))
            lo = f2i(fmin(fl, F(33)))
            hi = f2i(fmax(fh, F(-1))) - 1
            if lo > hi:
                lo, hi = 31, 0
            for i in range(3):
                mn[i] = mn[i] + st[i]
                mx[i] = mx[i] + st[i]
            rows[r] = (lo, hi)
        return rows

    @staticmethod
    def cols(rows, r0):
        m = 0
        for r in range(r0, r0 + 4):
            lo, hi = rows[r]
            if lo <= hi:
                m |= (0xF << (lo >> 3)) & (0xF >> (3 - (hi >> 3)))
        return m

    @staticmethod
    def centroid(rows, r0, startx):
        wy = [F(1), F(3), F(5), F(7)]
        px, py, n = [], [], 0
        for k in range(4):
            lo, hi = rows[r0 + k]
            xmin, xmax = max(lo - startx, 0), min(hi - startx, 7)
            c = max(xmax - xmin + 1, 0)
            px.append(F(xmin * 2 + c) * F(c))
            py.append(wy[k] * F(c))
            n += c
        return ((px[0] + px[1]) + px[2]) + px[3], ((py[0] + py[1]) + py[2]) + py[3], n

    def key(self, tri, cx, cy, n, bx, by, rng):
        d = self.depth[tri]
        scale = F(0.5) / F(n)
        px, py = cx * scale + F(bx), cy * scale + F(by)
        ray = bitsf(d[0]) * px + (bitsf(d[1]) * py + bitsf(d[2]))
        isq = F(1) / F(np.sqrt(ray + F(1)))
        return f2u(F(rng) * sat(isq))

    # ---- shading (shadeSample with lighting, RGBA8)
    def vertex_color(self, vid):
        c = self.sc.colors[vid]
        if self.sc.color_format == 0:
            return decode_rgba8(int(c))
        return [F(v) for v in np.asarray(c, np.float32)]

    def shade(self, tri, prim, px, py):
        d = self.depth[tri]
        b = self.bary[tri]
        fx, fy = F(px), F(py)
        inv = bitsf(d[0]) * fx + (bitsf(d[1]) * fy + bitsf(d[2]))
        ray = F(1) / inv
        e0 = bitsf(b[0]) * fx + (bitsf(b[1]) * fy + bitsf(b[2]))
        e1 = bitsf(b[4]) * fx + (bitsf(b[5]) * fy + bitsf(b[6]))
        b0 = e0 * ray - bitsf(b[3])
        b1 = e1 * ray - bitsf(b[7])
        flags, inst = int(d[3]) & 0xFFFF, int(d[3]) >> 16
        col = [F(1)] * 4
        if flags & 0x200 and self.sc.instance_colors is not None:  # INST_HAS_COLOR
            col = decode_rgba8(int(self.sc.instance_colors[inst]))
        if flags & 0x001:  # INST_HAS_VERTEX_COLORS
            q, second = tri >> 1, tri & 1
            v = self.verts[q]
            c0, c1, c2 = (self.vertex_color(int(v[0])), self.vertex_color(int(v[1 + second])),
                          self.vertex_color(int(v[2 + second])))
            wgt = (F(1) - b0) - b1
            col = [col[j] * (wgt * c0[j] + (b0 * c1[j] + b1 * c2[j])) for j in range(4)]
        if self.sc.tri_opacity is not None:
            col[3] = col[3] * F(self.sc.tri_opacity[prim])
        if col[3] == 0:
            return 0, inv
        n = int(self.normals[tri])
        s511 = F(1) / F(511)
        nrm = [(F(float((n >> (10 * i)) & 0x3FF)) - F(512)) * s511 for i in range(3)]
        dn = ((-self.sun_dir[0]) * nrm[0] + (-self.sun_dir[1]) * nrm[1]) + (-self.sun_dir[2]) * nrm[2]
        light = fmax(F(0), dn * F(0.7) + F(0.3))
        for ch in range(3):
            c = col[ch]
            lin = (F(1) / F(12.92)) * c if c < F(0.04045) else \
                pow_series((c + F(0.055)) * (F(1) / F(1.055)), F(2.4))
            amb = self.amb_color[ch] * self.amb_power
            dif = (self.sun_color[ch] * self.sun_power) * light
            v = lin * (amb + dif)
            srgb = F(12.92) * v if v < F(0.0031308) else \
                F(1.055) * pow_series(v, F(1) / F(2.4)) - F(0.055)
            col[ch] = sat(srgb)
        enc = f2u(col[0] * F(255)) | (f2u(col[1] * F(255)) << 8) | (f2u(col[2] * F(255)) << 16) | \
            (f2u(col[3] * F(255)) << 24)
        return enc, inv

    # ---- 3-deep window (reduceSample / finishReduceSamples)
    def reduce_pixel(self, samples):
        """samples: [(color, depth, segment)] in list order -> (rgba, invalid)"""
        vis = bool(self.flags & 8)
        additive = bool(self.flags & 2)
        D = 4 if vis else 3
        dep = [F(999999999.0)] * 4
        col = [0, 0, 0]
        st = {"trans": F(1), "out": [F(0)] * 3}

        def blend(c):
            cur = decode_rgba8(c)
            if additive:
                st["out"] = [st["out"][j] + cur[j] * cur[3] for j in range(3)]
            else:
                st["out"] = [st["out"][j] + (cur[j] * cur[3]) * st["trans"] for j in range(3)]
                st["trans"] = st["trans"] * (F(1) - cur[3])

        def swap_slots(a, b):
            dep[a], dep[b] = dep[b], dep[a]
            if a < 3 and b < 3:
                col[a], col[b] = col[b], col[a]

        invalid = False
        last_seg = None
        for color, depth, seg in samples:
            if last_seg is not None and seg != last_seg:
                st["out"] = [sat(v) for v in st["out"]]
            last_seg = seg
            skip = False
            if depth > dep[0]:
                color, col[0] = col[0], color
                depth, dep[0] = dep[0], depth
                if dep[0] > dep[1]:
                    swap_slots(0, 1)
                    if dep[1] > dep[2]:
                        swap_slots(1, 2)
                        i = 3
                        while i < D and dep[i - 1] > dep[i]:
                            swap_slots(i - 1, i)
                            i += 1
                        if D == 4 and i == D:
                            invalid = True
                            st["out"] = [F(1), F(0), F(0)]
                            st["trans"] = F(0)
                            skip = True
            if skip:
                continue
            for i in range(D - 1, 0, -1):
                dep[i] = dep[i - 1]
            dep[0] = depth
            if col[2] != 0:
                blend(col[2])
            col[2], col[1], col[0] = col[1], col[0], color
        if last_seg is not None:
            st["out"] = [sat(v) for v in st["out"]]
        for i in (2, 1, 0):
            if col[i] != 0:
                blend(col[i])
        rgba = [sat(st["out"][j] + st["trans"] * self.bg[j]) for j in range(3)] + [F(1)]
        return rgba, invalid

    # ---- one bin
    def bin_tris(self, b):
        o = self.o
        n = o["bin_count"]
        c = o["bin_counters"]
        tris = []
        for e in o["bin_quads"][c[n + b]:c[n + b] + c[b]]:
            q = int(e) & 0x0FFFFFFF
            for second in (0, 1):
                if not (int(e) >> (30 + second)) & 1:
                    tris.append((q * 2 + second, int(self.src[q]) * 2 + second))
        for t in o["bin_tris"][c[4 * n + b]:c[4 * n + b] + c[3 * n + b]]:
            t = int(t)
            tris.append((t, int(self.src[t >> 1]) * 2 + (t & 1)))
        return tris, int(c[3 * n + b]) + 2 * int(c[b])

    def render(self, low_high_threshold=1024):
        img = np.zeros((self.h, self.w, 4), np.float32)
        order = {}
        invalid = 0
        for b in range(self.o["bin_count"]):
            bin_x, bin_y = (b % self.bcx) * 32, (b // self.bcx) * 32
            tris, num = self.bin_tris(b)
            for r in range(32):
                for x in range(32):
                    if bin_x + x < self.w and bin_y + r < self.h:
                        img[bin_y + r, bin_x + x] = [sat(v) for v in self.bg] + [1.0]
            if num == 0:
                continue
            high = num >= low_high_threshold
            halfblocks = []  # (hx, hy, sorted [(tri, prim, rows)])
            if not high:
                rows = [self.rows(t, bin_x, bin_y, 8) for t, _ in tris]
                lists = [[] for _ in range(16)]
                for i, (t, p) in enumerate(tris):
                    for brow in range(4):
                        m = self.cols(rows[i], brow * 8) | self.cols(rows[i], brow * 8 + 4)
                        for bc in range(4):
                            if m >> bc & 1:
                                lists[brow * 4 + bc].append(i)
                if max(len(l) for l in lists) > 256:
                    high = True
                else:
                    for blk in range(16):
                        brow, bc = blk >> 2, blk & 3
                        ent = []
                        for i in lists[blk]:
                            t, p = tris[i]
                            cx0, cy0, n0 = self.centroid(rows[i], brow * 8, bc * 8)
                            cx1, cy1, n1 = self.centroid(rows[i], brow * 8 + 4, bc * 8)
                            k = self.key(t, cx0 + cx1, cy0 + cy1, n0 + n1, bin_x + bc * 8, bin_y + brow * 8,
                                         0x3FFFFE) if n0 + n1 else 0
                            ent.append((k, p, i))
                        ent.sort(key=(lambda e: (e[0], e[1])) if len(ent) > 3 else (lambda e: e[1]))
                        lst = [(tris[i][0], tris[i][1], rows[i]) for _, _, i in ent]
                        halfblocks.append((bc, brow * 2, lst))
                        halfblocks.append((bc, brow * 2 + 1, lst))
            if high:
                rows = [self.rows(t, bin_x, bin_y, 4) for t, _ in tris]
                lists = [[] for _ in range(32)]
                for i in range(len(tris)):
                    for hr in range(8):
                        m = self.cols(rows[i], hr * 4)
                        for c in range(4):
                            if m >> c & 1:
                                lists[hr * 4 + c].append(i)
                for hb in range(32):
                    hr, hc = hb >> 2, hb & 3
                    ent = []
                    for i in lists[hb]:
                        t, p = tris[i]
                        cx, cy, n = self.centroid(rows[i], hr * 4, hc * 8)
                        k = self.key(t, cx, cy, n, bin_x + hc * 8, bin_y + hr * 4, 0x7FFFE) if n else 0
                        ent.append((k, p, i))
                    ent.sort(key=lambda e: (e[0], e[1]))
                    halfblocks.append((hc, hr, [(tris[i][0], tris[i][1], rows[i]) for _, _, i in ent]))
            for hx, hy, lst in halfblocks:
                samples = {pl: [] for pl in range(32)}
                offset = 0
                for t, p, rows_t in lst:
                    rank = 0
                    for k in range(4):
                        lo, hi = rows_t[hy * 4 + k]
                        for x in range(max(lo - hx * 8, 0), min(hi - hx * 8, 7) + 1):
                            pl = k * 8 + x
                            px, py = bin_x + hx * 8 + x, bin_y + hy * 4 + k
                            c, d = self.shade(t, p, px, py)
                            samples[pl].append((c, d, (offset + rank) >> 8, p))
                            rank += 1
                    offset += rank
                for pl in range(32):
                    px, py = bin_x + hx * 8 + (pl & 7), bin_y + hy * 4 + (pl >> 3)
                    if px >= self.w or py >= self.h:
                        continue
                    rgba, inv = self.reduce_pixel([s[:3] for s in samples[pl]])
                    img[py, px] = rgba
                    invalid += inv
                    order[(py, px)] = [s[3] for s in samples[pl]]
        return img, order, invalid
