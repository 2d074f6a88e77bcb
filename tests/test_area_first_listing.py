"""The area kernel's deduplication rule, restated on the CPU over oracle rasters.

An edge of polygon O is listed by every pixel it passes, so the window
searched for the edges that may cross a segment meets it several times. The
kernel counts a crossing only at the edge's first listing in the window's own
enumeration order (farm_gb300/csrc/area.cu: seg_window, row_cols,
for_candidate_edges, first_listing, k_edge_pix_sort). Here the same window
arithmetic (IEEE double, as the kernel's explicit roundings) and the same rule,
with a ring of the last 16 rows and row_cols beyond it, run over dense spiky rasters and
random segments; every edge listed in a window must be accepted exactly once.
"""
import math

import numpy as np
import pytest

from farm_gb300 import polygons as P
from oracle import oracle as O

K_ROW_CACHE = 16


def double_to_int(v):
    vi = int(v)  # truncation toward zero, as the C cast
    if abs(1.0 * (vi + 1) - v) < 0.00000001:
        vi += 1
    return vi


def offset_x(mbr, step, dim, v):
    x = double_to_int((v - mbr[0]) / step)
    return min(max(x, 0), dim - 1)


def offset_y(mbr, step, dim, v):
    y = double_to_int((v - mbr[1]) / step)
    return min(max(y, 0), dim - 1)


def show_status(s, cc=16):
    return 0 if s == 0 else (2 if s == cc - 1 else 1)


class Ras:
    def __init__(self, r):
        a = r.arrays()
        self.mbr, self.dimx, self.dimy = a["mbr"], a["dimx"], a["dimy"]
        self.sx_, self.sy_ = float(a["step"][0]), float(a["step"][1])
        self.status, self.off, self.seq = a["status"], a["offset"], a["seq"]
        # edge -> ascending pixel ids, from the same (pixel, sequence) walk
        lists = {}
        for pid in range(self.dimx * self.dimy):
            for q in range(int(self.off[pid]), int(self.off[pid + 1])):
                s0, ln = int(self.seq[q, 0]), int(self.seq[q, 1])
                for k in range(ln):
                    lists.setdefault(s0 + k, []).append(pid)
        self.lists = {f: sorted(v) for f, v in lists.items()}


def seg_window(R, x0, y0, x1, y1):
    mnx, mxx, mny, mxy = min(x0, x1), max(x0, x1), min(y0, y1), max(y0, y1)
    m = R.mbr
    if mxx < m[0] or mnx > m[2] or mxy < m[1] or mny > m[3]:
        return None
    sx = max(offset_x(m, R.sx_, R.dimx, mnx) - 1, 0)
    ex = min(offset_x(m, R.sx_, R.dimx, mxx) + 1, R.dimx - 1)
    sy = max(offset_y(m, R.sy_, R.dimy, mny) - 1, 0)
    ey = min(offset_y(m, R.sy_, R.dimy, mxy) + 1, R.dimy - 1)
    return (x0, y0, x1, y1, sx, ex, sy, ey)


def row_cols(R, w, y):
    x0, y0, x1, y1, sx, ex, sy, ey = w
    if y1 == y0:
        return True, sx, ex
    ylo = R.mbr[1] + float(y - 1) * R.sy_
    yhi = R.mbr[1] + float(y + 2) * R.sy_
    dy = y1 - y0
    ta, tb = (ylo - y0) / dy, (yhi - y0) / dy
    if ta > tb:
        ta, tb = tb, ta
    ta, tb = max(ta, 0.0), min(tb, 1.0)
    if ta > tb:
        return False, sx, ex
    dx = x1 - x0
    xa_, xb_ = x0 + ta * dx, x0 + tb * dx
    if xa_ > xb_:
        xa_, xb_ = xb_, xa_
    ca = offset_x(R.mbr, R.sx_, R.dimx, xa_) - 1
    cb = offset_x(R.mbr, R.sx_, R.dimx, xb_) + 1
    return True, max(ca, sx), min(cb, ex)


def enumerate_window(R, w):
    """(pid, xa, q, f) in for_candidate_edges' order, each with the row ring
    as it stood when that listing was met."""
    out, cache = [], {}
    _, _, _, _, sx, ex, sy, ey = w
    for y in range(sy, ey + 1):
        ok, xa, xb = row_cols(R, w, y)
        cache[y & (K_ROW_CACHE - 1)] = (xa, xb) if ok else (1, 0)
        if not ok:
            continue
        for x in range(xa, xb + 1):
            pid = y * R.dimx + x
            if show_status(R.status[pid]) != 1:
                continue
            for q in range(int(R.off[pid]), int(R.off[pid + 1])):
                s0, ln = int(R.seq[q, 0]), int(R.seq[q, 1])
                for k in range(ln):
                    out.append((pid, xa, q, s0 + k, dict(cache)))
    return out


def first_listing(R, w, cache, pid, xa, q, f):
    sy = w[6]
    py = pid // R.dimx
    self_n = 0
    for r in R.lists[f]:
        if r > pid:
            break
        if r == pid:
            self_n += 1
            continue
        ry, rx = r // R.dimx, r % R.dimx
        if ry < sy or show_status(R.status[r]) != 1:
            continue
        if ry == py:
            if rx >= xa:
                return False
            continue
        if ry > py - K_ROW_CACHE:
            cxa, cxb = cache[ry & (K_ROW_CACHE - 1)]
        else:
            ok, cxa, cxb = row_cols(R, w, ry)
            if not ok:
                continue
        if cxa <= rx <= cxb:
            return False
    if self_n > 1:
        for p in range(int(R.off[pid]), q):
            s0, ln = int(R.seq[p, 0]), int(R.seq[p, 1])
            if s0 <= f < s0 + ln:
                return False
    return True


@pytest.mark.parametrize("seed,n_hi,vpr", [(71, 3000, 10), (72, 20000, 10), (73, 8000, 4)])
def test_first_listing_accepts_each_listed_edge_once(host_built, seed, n_hi, vpr):
    prm = P.StarParams(dom_hi=1.0, r_lo=0.3, r_hi=0.4, n_lo=n_hi // 2, n_hi=n_hi)
    ps = P.generate(prm, seed, 2)
    rng = np.random.default_rng(seed)
    checked = multi = 0
    for k in range(ps.n):
        R = Ras(O.Raster(ps.ring(k), vpr))
        m = R.mbr
        cx, cy = 0.5 * (m[0] + m[2]), 0.5 * (m[1] + m[3])
        span = max(m[2] - m[0], m[3] - m[1])
        for i in range(60):
            # short segments (a pixel or two) and long ones across the raster,
            # some axis-parallel, with float32 endpoints as the kernel's
            ln = span * (0.02 if i % 3 == 0 else (0.15 if i % 3 == 1 else 1.2))
            a = rng.uniform(0, 2 * math.pi)
            if i % 10 == 0:
                a = 0.0
            elif i % 10 == 5:
                a = math.pi / 2
            px = cx + rng.uniform(-0.5, 0.5) * span
            py = cy + rng.uniform(-0.5, 0.5) * span
            x0, y0 = float(np.float32(px)), float(np.float32(py))
            x1, y1 = float(np.float32(px + ln * math.cos(a))), float(np.float32(py + ln * math.sin(a)))
            w = seg_window(R, x0, y0, x1, y1)
            if w is None:
                continue
            listed = enumerate_window(R, w)
            counts = {}
            for pid, xa, q, f, cache in listed:
                if first_listing(R, w, cache, pid, xa, q, f):
                    counts[f] = counts.get(f, 0) + 1
            edges = {f for _, _, _, f, _ in listed}
            assert set(counts) == edges and all(c == 1 for c in counts.values()), (k, i)
            checked += len(edges)
            multi += len(listed) - len(edges)
    assert checked > 1000 and multi > 1000  # many edges, many repeated listings
