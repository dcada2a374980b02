"""A second, independent transcription of the reference's step in Python.

Pure-Python loops over numpy float32 scalars (each operation rounds to f32,
as Rust's f32 arithmetic does), used only on small cases to cross-check the
C++ oracle's transcription of:
  field_2d.rs:304-339 (new, discretize), 386-516 (both queries),
  838-846 / 905-921 (set_object_location, lazy_update), 926-1014 (helpers),
  bird.rs:39-154 (Bird::step), and Philox4x32-10 (SC'11) for the jitter.
"""
import numpy as np

f32 = np.float32
M32 = 0xFFFFFFFF


def philox4x32_10(ctr, key):
    c = [int(v) & M32 for v in ctr]
    k0, k1 = int(key[0]) & M32, int(key[1]) & M32
    for r in range(10):
        if r:
            k0 = (k0 + 0x9E3779B9) & M32
            k1 = (k1 + 0xBB67AE85) & M32
        p0 = 0xD2511F53 * c[0]
        p1 = 0xCD9E8D57 * c[2]
        c = [((p1 >> 32) ^ c[1] ^ k0) & M32, p1 & M32, ((p0 >> 32) ^ c[3] ^ k1) & M32, p0 & M32]
    return c


def unit(u):
    return f32(u >> 8) * f32(1.0 / 16777216.0)


def as_i32(v):
    v = float(v)
    if v != v:
        return 0
    return int(max(min(v, 2147483647.0), -2147483648.0))


def t_transform(n, size):
    # Rust i32 % truncates toward zero
    r = abs(n) % size
    r = r if n >= 0 else -r
    return r if n >= 0 else r + size


def toroidal_transform(v, dim):
    if v >= f32(0) and v < dim:
        return v
    r = f32(np.fmod(v, dim))
    if r < f32(0):
        r = f32(r + dim)
    return r


def toroidal_distance(a, b, dim):
    if abs(f32(a - b)) <= f32(dim / f32(2)):
        return f32(a - b)
    d = f32(toroidal_transform(a, dim) - toroidal_transform(b, dim))
    if f32(d * f32(2)) > dim:
        return f32(d - dim)
    if f32(d * f32(2)) < -dim:
        return f32(d + dim)
    return d


def distance(x1, y1, x2, y2, w, h, tor):
    if tor:
        dx = toroidal_distance(x1, x2, w)
        dy = toroidal_distance(y1, y2, h)
    else:
        dx, dy = f32(x1 - x2), f32(y1 - y2)
    return f32(np.sqrt(f32(f32(dx * dx) + f32(dy * dy))))


class PyField:
    def __init__(self, w, h, d, tor=True, wrap=False):
        self.w, self.h, self.d, self.tor = f32(w), f32(h), f32(d), tor
        self.wrap = bool(tor and wrap)  # true-torus query range (not in the reference)
        self.max_x = as_i32(np.ceil(f32(self.w / self.d)))
        self.max_y = as_i32(np.ceil(f32(self.h / self.d)))
        self.dw, self.dh = self.max_x + 1, self.max_y + 1
        self.read = [[] for _ in range(self.dw * self.dh)]
        self.write = [[] for _ in range(self.dw * self.dh)]

    def disc(self, x, y):
        return as_i32(np.floor(f32(f32(x) / self.d))), as_i32(np.floor(f32(f32(y) / self.d)))

    def set(self, bird, lx, ly):
        cx, cy = self.disc(lx, ly)
        self.write[cx * self.dh + cy].append(bird)

    def lazy_update(self):
        self.read, self.write = self.write, [[] for _ in range(self.dw * self.dh)]

    def _range(self, x, y, dist):
        dd = as_i32(np.floor(f32(f32(dist) / self.d)))
        cx, cy = self.disc(x, y)
        a, b, c, e = cx - dd, cx + dd, cy - dd, cy + dd
        if self.tor and not self.wrap:
            a, b, c, e = max(0, a), min(b, self.max_x - 1), max(0, c), min(e, self.max_y - 1)
        elif self.wrap:
            if 2 * dd + 1 >= self.max_x:
                a, b = 0, self.max_x - 1
            if 2 * dd + 1 >= self.max_y:
                c, e = 0, self.max_y - 1
        return a, b, c, e

    def check_circle(self, bx, by, lx, ly, dis):
        nw = (f32(f32(bx) * self.d), f32(f32(by) * self.d))
        ne = (nw[0], min(f32(nw[1] + self.d), self.h))
        sw = (min(f32(nw[0] + self.d), self.w), nw[1])
        se = (sw[0], ne[1])
        ds = [distance(p[0], p[1], lx, ly, self.w, self.h, self.tor) for p in (nw, ne, sw, se)]
        if all(v <= dis for v in ds):
            return 1
        if all(v > dis for v in ds):
            return -1
        return 0

    def query(self, kind, x, y, dist):
        out = []
        dist = f32(dist)
        if dist <= f32(0):
            return out
        a, b, c, e = self._range(x, y, dist)
        for i in range(a, b + 1):
            for j in range(c, e + 1):
                bx, by = t_transform(i, self.max_x), t_transform(j, self.max_y)
                bag = self.read[bx * self.dh + by]
                if kind == 0:
                    out.extend(bag)
                    continue
                chk = self.check_circle(bx, by, f32(x), f32(y), dist)
                for el in bag:
                    if chk == 1 or (chk == 0 and distance(f32(x), f32(y), el[1], el[2], self.w,
                                                          self.h, self.tor) <= dist):
                        out.append(el)
        return out


def bird_step(fld, me, kind, radius, weights, jump, seed, step):
    """bird.rs:39-154; me = (id, x, y, dx, dy) as f32; returns the new tuple."""
    coh, avo, con, rnd, mom = (f32(v) for v in weights)
    jump = f32(jump)
    vec = fld.query(kind, me[1], me[2], radius)
    w, h = fld.w, fld.h
    av = co = ra = cs = (f32(0), f32(0))
    if vec:
        xa = ya = xc = yc = xs = ys = f32(0)
        count = 0
        for el in vec:
            if el[0] != me[0]:
                dx = toroidal_distance(me[1], el[1], w)
                dy = toroidal_distance(me[2], el[2], h)
                count += 1
                sq = f32(f32(dx * dx) + f32(dy * dy))
                q = f32(f32(sq * sq) + f32(1))
                xa = f32(xa + f32(dx / q))
                ya = f32(ya + f32(dy / q))
                xc, yc = f32(xc + dx), f32(yc + dy)
                xs, ys = f32(xs + el[3]), f32(ys + el[4])
        if count > 0:
            c = f32(count)
            xa, ya, xc, yc, xs, ys = (f32(v / c) for v in (xa, ya, xc, yc, xs, ys))
            cs = (f32(xs / c), f32(ys / c))
        else:
            cs = (xs, ys)
        av = (f32(f32(400) * xa), f32(f32(400) * ya))
        co = (f32(-xc / f32(10)), f32(-yc / f32(10)))
        o = philox4x32_10([me[0], step & M32, step >> 32, 0], [seed & M32, seed >> 32])
        xr = f32(f32(unit(o[0]) * f32(2)) - f32(1))
        yr = f32(f32(unit(o[1]) * f32(2)) - f32(1))
        sq = f32(np.sqrt(f32(f32(xr * xr) + f32(yr * yr))))
        ra = (f32(f32(f32(0.05) * xr) / sq), f32(f32(f32(0.05) * yr) / sq))
    dx = f32(f32(f32(f32(f32(coh * co[0]) + f32(avo * av[0])) + f32(con * cs[0])) +
                 f32(rnd * ra[0])) + f32(mom * me[3]))
    dy = f32(f32(f32(f32(f32(coh * co[1]) + f32(avo * av[1])) + f32(con * cs[1])) +
                 f32(rnd * ra[1])) + f32(mom * me[4]))
    dis = f32(np.sqrt(f32(f32(dx * dx) + f32(dy * dy))))
    if dis > f32(0):
        dx = f32(f32(dx / dis) * jump)
        dy = f32(f32(dy / dis) * jump)
    nx = toroidal_transform(f32(me[1] + dx), w)
    ny = toroidal_transform(f32(me[2] + dy), w)
    return (me[0], nx, ny, dx, dy)


def flock_step(fld, kind, radius, weights, jump, seed, step):
    """One Schedule::step in read-buffer iteration order, then lazy_update."""
    agents = [b for bag in fld.read for b in bag]
    for me in agents:
        nb = bird_step(fld, me, kind, radius, weights, jump, seed, step)
        fld.set(nb, nb[1], nb[2])
    fld.lazy_update()
