"""Pure-Python restatement of euc 0.6.0's triangle pipeline (test
infrastructure only; small scenes only: every pixel step is a Python loop).

It is written independently of euc_oracle.cpp, directly from euc's source,
with numpy float32 scalars (IEEE single, no FMA): agreement of the two
restatements on random scenes pins the C++ oracle against slips of either.
PARITY UNPINNED: neither has been checked against euc's own output.

Citations are file:line in euc 0.6.0.
"""
import math

import numpy as np

from euc_gb300 import abi

F = np.float32
EPS = F(1.1920928955078125e-07)  # core::f32::EPSILON
U64 = (1 << 64) - 1


def fmin(a, b):  # f32::min: the non-NaN operand wins
    return b if math.isnan(a) else (a if math.isnan(b) else (a if a < b else b))


def fmax(a, b):
    return b if math.isnan(a) else (a if math.isnan(b) else (a if a > b else b))


def as_usize(v):  # saturating `as usize`
    if math.isnan(v) or v < 1.0:
        return 0
    if v >= 18446744073709551616.0:
        return U64
    return int(v)


def as_u8(v):
    if math.isnan(v) or v < 1.0:
        return 0
    if v >= 255.0:
        return 255
    return int(v)


def fract(v):
    return F(v - np.trunc(v))


def rem_euclid(x, m):
    r = F(np.fmod(x, m))
    return F(r + abs(m)) if r < 0 else r


def clamp(v, lo, hi):
    return lo if v < lo else (hi if v > hi else v)


# ---- example-shader maths (op order documented in include/euc_gb300.h) ----
def mat4_vec4(m, v):
    return [F(F(F(F(m[r * 4] * v[0]) + F(m[r * 4 + 1] * v[1])) + F(m[r * 4 + 2] * v[2])) + F(m[r * 4 + 3] * v[3]))
            for r in range(4)]


def sdot(a, b):
    return F(F(F(a[0] * b[0]) + F(a[1] * b[1])) + F(a[2] * b[2]))


def normalize(a):
    ln = F(np.sqrt(sdot(a, a)))
    return [F(a[0] / ln), F(a[1] / ln), F(a[2] / ln)]


class Tex:
    def __init__(self, s):  # s: (array, filter, wrap, texel_div)
        self.arr, self.filter, self.wrap, self.div = s
        self.h, self.w = self.arr.shape[0], self.arr.shape[1]

    def read(self, x, y):
        if self.arr.dtype == np.float32:
            v = F(self.arr[y, x])
            return [v, v, v, v]
        return [F(F(int(c)) / F(self.div)) for c in self.arr[y, x]]

    def sample(self, u, v):
        def wrap(e):
            if self.wrap == abi.WRAP_CLAMP:
                return fmin(fmax(e, F(0)), F(1))
            if self.wrap == abi.WRAP_TILE:
                return rem_euclid(e, F(1))
            if self.wrap == abi.WRAP_MIRROR:
                return F(F(1) - rem_euclid(e, F(1))) if rem_euclid(e, F(2)) >= 1.0 else rem_euclid(e, F(1))
            return e
        u, v = wrap(F(u)), wrap(F(v))
        w, h = self.w, self.h
        if self.filter == abi.FILTER_NEAREST:  # math.rs:51-53
            return self.read(min(as_usize(fmax(F(u * F(w)), F(0))), w - 1), min(as_usize(fmax(F(v * F(h)), F(0))), h - 1))
        itx, ity = F(fract(u) * F(w)), F(fract(v) * F(h))  # linear.rs:30-66
        px, py = as_usize(np.trunc(itx)), as_usize(np.trunc(ity))
        fx, fy = fract(itx), fract(ity)
        p0x, p0y, p1x, p1y = min(px, w - 1), min(py, h - 1), min(px + 1, w - 1), min(py + 1, h - 1)
        t00, t10, t01, t11 = self.read(p0x, p0y), self.read(p1x, p0y), self.read(p0x, p1y), self.read(p1x, p1y)
        out = []
        for i in range(4):
            t0 = F(F(t00[i] * F(F(1) - fy)) + F(t01[i] * fy))
            t1 = F(F(t10[i] * F(F(1) - fy)) + F(t11[i] * fy))
            out.append(F(F(t0 * F(F(1) - fx)) + F(t1 * fx)))
        return out


def _f(v, off, i=0):
    return F(np.frombuffer(v[off + 4 * i: off + 4 * i + 4].tobytes(), dtype=np.float32)[0])


class Shader:
    """vertex / fragment / pack of one example pipeline kind."""

    def __init__(self, kind, u, lay, texs):
        self.kind, self.u, self.lay, self.texs = kind, u, lay, texs

    def vertex(self, v):
        u, l = self.u, self.lay
        pos = [_f(v, l.position, i) for i in range(3)]
        if self.kind == abi.SHADER_VCOLOR:
            p = pos + [_f(v, l.position, 3)]
            return mat4_vec4(list(u.mvp), p), [F(F(int(c)) / F(255)) for c in v[l.color:l.color + 4]]
        if self.kind in (abi.SHADER_FLAT, abi.SHADER_SHADOW):
            return mat4_vec4(list(u.mvp), pos + [F(1)]), [F(0)]
        if self.kind == abi.SHADER_GOURAUD:
            clip = mat4_vec4(list(u.mvp), pos + [F(1)])
            n = normalize(mat4_vec4(list(u.model), [_f(v, l.normal, i) for i in range(3)] + [F(0)])[:3])
            lam = fmax(sdot(n, [F(x) for x in u.to_light]), F(0))
            k = F(F(u.ambient) + F(lam * F(u.diffuse)))
            return clip, [F(F(c) * k) for c in u.color]
        if self.kind == abi.SHADER_TEXTURED:
            return mat4_vec4(list(u.mvp), pos + [F(1)]), [_f(v, l.uv, 0), _f(v, l.uv, 1)]
        # PHONG (examples/teapot.rs:81-96)
        ns = F(u.normal_sign)
        wpos = mat4_vec4(list(u.model), pos + [F(1)])
        wnorm = mat4_vec4(list(u.model), [F(_f(v, l.normal, i) * ns) for i in range(3)] + [F(0)])
        lvp = mat4_vec4(list(u.light_vp), wpos[:3] + [F(1)])
        clip = mat4_vec4(list(u.proj), mat4_vec4(list(u.view), wpos))
        uv = [_f(v, l.uv, 0), _f(v, l.uv, 1)] if l.uv >= 0 else [F(0), F(0)]
        return clip, wpos[:3] + wnorm[:3] + [F(lvp[0] / lvp[3]), F(lvp[1] / lvp[3]), F(lvp[2] / lvp[3])] + uv

    def fragment(self, vd):
        u = self.u
        if self.kind == abi.SHADER_VCOLOR:
            return list(vd)
        if self.kind == abi.SHADER_FLAT:
            return [F(c) for c in u.color]
        if self.kind == abi.SHADER_SHADOW:
            return [F(0)]
        if self.kind == abi.SHADER_GOURAUD:
            return [vd[0], vd[1], vd[2], F(1)]
        if self.kind == abi.SHADER_TEXTURED:
            return self.texs["tex"].sample(vd[0], vd[1])
        n = normalize(vd[3:6])  # examples/teapot.rs:98-131
        cam = normalize([F(F(u.cam_pos[i]) - vd[i]) for i in range(3)])
        ld = normalize([F(vd[i] - F(u.light_pos[i])) for i in range(3)])
        surf = self.texs["tex"].sample(vd[9], vd[10]) if "tex" in self.texs else [F(c) for c in u.surf_color]
        nl = [F(-x) for x in ld]
        diffuse = F(fmax(sdot(n, nl), F(0)) * F(0.5))
        d = sdot(nl, n)
        dd = F(d + d)
        r = [F(nl[i] - F(n[i] * dd)) for i in range(3)]
        nc = [F(-x) for x in cam]
        spec = F(F(np.power(fmax(sdot(r, nc), F(0)), F(30))) * F(3))
        lit = True
        if "shadow" in self.texs:
            su = F(F(F(vd[6] * F(1)) * F(0.5)) + F(0.5))
            sv = F(F(F(vd[7] * F(-1)) * F(0.5)) + F(0.5))
            lit = vd[8] < F(self.texs["shadow"].sample(su, sv)[0] + F(0.0001))
        light = F(F(u.ambient) + (F(diffuse + spec) if lit else F(0)))
        return [F(s * light) for s in surf]

    def pack(self, c):
        if self.kind == abi.SHADER_TEXTURED or self.kind == abi.SHADER_SHADOW:
            return c
        if self.kind == abi.SHADER_PHONG:
            return F(fmin(fmax(c, F(0)), F(1)) * F(255))
        return F(c * F(255))


def render(desc, shader, verts, nverts, stride, idx, pixel, pfmt, depth):
    """Pipeline::render on numpy targets (modified in place); returns
    (status, candidates)."""
    uses_depth = desc.depth_test != abi.TEST_NONE or bool(desc.depth_write)
    if not desc.pixel_write and not uses_depth:
        return abi.OK, 0
    psize = (pixel.shape[1], pixel.shape[0]) if pixel is not None else (0, 0)
    dsize = (depth.shape[1], depth.shape[0]) if depth is not None else (0, 0)
    if desc.pixel_write and not uses_depth:
        size = psize
    elif not desc.pixel_write:
        size = dsize
    else:
        if psize != dsize:
            return abi.ERR_SIZE_MISMATCH, 0
        size = psize
    stream = list(idx) if idx is not None else list(range(nverts))
    if any(int(i) >= nverts for i in stream):
        return abi.ERR_INDEX_OOB, 0
    vout = [shader.vertex(verts[int(i) * stride:(int(i) + 1) * stride]) for i in stream]
    level = min(desc.aa_level, 6)
    W, H = size
    if desc.band_rows == abi.BANDS_PAR:  # pipeline.rs:328-330
        gr = 20000 * (1 << level) // max(W, 1)
        if gr == 0:
            return abi.ERR_BAND, 0
        if H // gr == 0:
            if desc.flags & abi.FLAG_PAR_EMPTY:
                return abi.OK, 0
            gr = max(H, 1)
    else:
        gr = min(desc.band_rows, max(H, 1))
    cand = 0
    row = 0
    while row < H:
        cand += _render_band(desc, shader, vout, (W, H), row, min(row + gr, H), level, pixel, pfmt, depth)
        row += gr
    return abi.OK, cand


def _render_band(desc, sh, vout, size, row0, row1, level, pixel, pfmt, depth):
    W, H = size
    tmin, tmax = (0, row0), (W, row1)
    sx, sy = F(W), F(H)
    flip = F(-1) if desc.y_axis == abi.Y_UP else F(1)
    msaa = {}  # (cx, cy) -> (primitive_count, fragment)
    msaa_div = F(F(1) / F(1 << level))
    pc = 0
    cand = 0
    for t in range(len(vout) // 3):
        pc += 1  # begin_primitive
        hom = [[F(vout[3 * t + k][0][0] * F(1)), F(vout[3 * t + k][0][1] * flip), vout[3 * t + k][0][2],
                vout[3 * t + k][0][3]] for k in range(3)]
        vd = [vout[3 * t + k][1] for k in range(3)]
        eu = [[F(h[0] / h[3]), F(h[1] / h[3]), F(h[2] / h[3])] for h in hom]
        a = [F(eu[1][i] - eu[0][i]) for i in range(3)]
        b = [F(eu[2][i] - eu[0][i]) for i in range(3)]
        winding = F(F(a[0] * b[1]) - F(a[1] * b[0]))
        if desc.cull != abi.CULL_NONE:
            if F(winding * (F(1) if desc.cull == abi.CULL_BACK else F(-1))) < 0:
                continue
        if winding >= 0:
            hom, eu, vd = hom[::-1], eu[::-1], vd[::-1]
        A, B, Cc = [hom[0][0], hom[0][1], hom[0][3]], [hom[1][0], hom[1][1], hom[1][3]], [hom[2][0], hom[2][1], hom[2][3]]
        ca = [F(A[i] - Cc[i]) for i in range(3)]
        cb = [F(B[i] - Cc[i]) for i in range(3)]

        def cross(p, q):
            return [F(F(p[1] * q[2]) - F(p[2] * q[1])), F(F(p[2] * q[0]) - F(p[0] * q[2])),
                    F(F(p[0] * q[1]) - F(p[1] * q[0]))]
        n = cross(ca, cb)
        rec = F(F(1) / fmin(sdot(n, Cc), -EPS)) if sdot(n, n) > 0 else F(1)
        rows = [[F(e * rec) for e in r] for r in (cross(cb, Cc), cross(Cc, ca), n)]
        nd = [[F(F(2) / sx), F(0), F(-1)], [F(0), F(F(-2) / sy), F(1)], [F(0), F(0), F(1)]]
        M = [[F(F(F(rows[i][0] * nd[0][j]) + F(rows[i][1] * nd[1][j])) + F(rows[i][2] * nd[2][j])) for j in range(3)]
             for i in range(3)]
        scr = [[F(sx * F(F(e[0] * F(0.5)) + F(0.5))), F(sy * F(F(e[1] * F(-0.5)) + F(0.5)))] for e in eu]
        bmin = [clamp(as_usize(F(fmin(fmin(scr[0][k], scr[1][k]), scr[2][k]) + F(0))), tmin[k], tmax[k]) for k in (0, 1)]
        bmax = [clamp(as_usize(F(fmax(fmax(scr[0][k], scr[1][k]), scr[2][k]) + F(1))), tmin[k], tmax[k]) for k in (0, 1)]

        def wat(p0, p1):
            return [F(F(F(M[i][0] * p0) + F(M[i][1] * p1)) + F(M[i][2] * F(1))) for i in range(3)]
        o = wat(F(0), F(0))
        dx = [F(F(e - oo) * F(F(1) / F(1000))) for e, oo in zip(wat(F(1000), F(0)), o)]
        dy = [F(F(e - oo) * F(F(1) / F(1000))) for e, oo in zip(wat(F(0), F(1000)), o)]
        ys = [s[1] for s in scr]
        mny = fmin(fmin(ys[0], ys[1]), ys[2])
        if scr[0][1] == mny:
            by = [scr[0], scr[1], scr[2]] if scr[1][1] < scr[2][1] else [scr[0], scr[2], scr[1]]
        elif scr[1][1] == mny:
            by = [scr[1], scr[0], scr[2]] if scr[0][1] < scr[2][1] else [scr[1], scr[2], scr[0]]
        else:
            by = [scr[2], scr[0], scr[1]] if scr[0][1] < scr[1][1] else [scr[2], scr[1], scr[0]]

        def zc_ok(z):
            return (not desc.z_clip) or (F(desc.z_clip_min) <= z <= F(desc.z_clip_max))
        noclip = all(zc_ok(e[2]) for e in eu)
        zc = [h[2] for h in hom]

        def gv(xf, yf):
            w = [F(F(o[c] + F(dy[c] * yf)) + F(dx[c] * xf)) for c in range(3)]
            wu = [w[0], w[1], F(F(w[2] - w[0]) - w[1])]
            r = F(F(1) / w[2])
            wp = [F(e * r) for e in wu]
            return [F(F(F(vd[0][i] * wp[0]) + F(vd[1][i] * wp[1])) + F(vd[2][i] * wp[2])) for i in range(len(vd[0]))]

        for y in range(bmin[1], bmax[1]):
            ext = ((bmax[0] - bmin[0]) * (bmax[1] - bmin[1])) & U64
            yf = F(y)
            if ext < 128:
                xs, xe = bmin[0], bmax[0]
            else:
                Av, Bv, Cv = by
                ac = F(Av[0] + F(F(F(yf - Av[1]) / F(Cv[1] - Av[1])) * F(Cv[0] - Av[0])))
                if yf < Bv[1]:
                    e2 = F(Av[0] + F(F(F(yf - Av[1]) / F(Bv[1] - Av[1])) * F(Bv[0] - Av[0])))
                else:
                    e2 = F(Bv[0] + F(F(F(yf - Bv[1]) / F(Cv[1] - Bv[1])) * F(Cv[0] - Bv[0])))
                lo, hi = fmin(e2, ac), fmax(e2, ac)
                fl, ce = F(np.floor(lo)), F(np.ceil(hi))
                xs = as_usize(fl) if (fl >= F(bmin[0]) and fl < F(bmax[0])) else bmin[0]
                xe = as_usize(ce) if (ce >= F(bmin[0]) and ce < F(bmax[0])) else bmax[0]
            w = [F(F(o[c] + F(dy[c] * yf)) + F(dx[c] * F(xs))) for c in range(3)]
            for x in range(xs, xe):
                wu = [w[0], w[1], F(F(w[2] - w[0]) - w[1])]
                if wu[0] >= 0 and wu[1] >= 0 and wu[2] >= 0:
                    z = F(F(F(zc[0] * wu[0]) + F(zc[1] * wu[1])) + F(zc[2] * wu[2]))
                    if noclip or zc_ok(z):
                        cand += 1
                        ok = True
                        if desc.depth_test != abi.TEST_NONE:
                            old = depth[y, x]
                            ok = {abi.TEST_LESS: z < old, abi.TEST_EQUAL: z == old, abi.TEST_GREATER: z > old}[desc.depth_test]
                        if ok:
                            if desc.depth_write:
                                depth[y, x] = z
                            if desc.pixel_write:
                                if level == 0:
                                    frag = sh.fragment(gv(F(x), yf))
                                else:
                                    fxm = fract(F(F(x - tmin[0]) * msaa_div))
                                    fym = fract(F(F(y - tmin[1]) * msaa_div))
                                    px, py = (x - tmin[0]) >> level, (y - tmin[1]) >> level

                                    def coarse(cx, cy):
                                        e = msaa.get((cx, cy))
                                        if e is None or e[0] != pc:
                                            e = (pc, sh.fragment(gv(F(tmin[0] + (cx << level)), F(tmin[1] + (cy << level)))))
                                            msaa[(cx, cy)] = e
                                        return e[1]
                                    t00, t10, t01, t11 = coarse(px, py), coarse(px + 1, py), coarse(px, py + 1), coarse(px + 1, py + 1)
                                    frag = []
                                    for i in range(len(t00)):
                                        a0 = F(F(t00[i] * F(F(1) - fym)) + F(t01[i] * fym))
                                        a1 = F(F(t10[i] * F(F(1) - fym)) + F(t11[i] * fym))
                                        frag.append(F(F(a0 * F(F(1) - fxm)) + F(a1 * fxm)))
                                c = (list(frag) + [F(0)] * 4)[:4]
                                if desc.blend == abi.BLEND_ALPHA:  # src-over on the unpacked old pixel
                                    px = [int(v) for v in pixel[y, x, :]]
                                    if pfmt == abi.FMT_BGRA8:
                                        px = [px[2], px[1], px[0], px[3]]
                                    old = [F(F(px[i]) / F(255)) for i in range(3)]
                                    old.append(F(1) if pfmt == abi.FMT_RGB8 else F(F(px[3]) / F(255)))
                                    a = c[3]
                                    c = [F(F(c[i] * a) + F(old[i] * F(F(1) - a))) for i in range(4)]
                                ch = [as_u8(sh.pack(v)) for v in c]
                                if pfmt == abi.FMT_BGRA8:
                                    ch = [ch[2], ch[1], ch[0], ch[3]]
                                pixel[y, x, :] = ch[:pixel.shape[2]]
                w = [F(w[c] + dx[c]) for c in range(3)]
    return cand


def run_pass(frame, p, targets):
    """Runs one scenes.PassSpec against host targets (dict name -> array)."""
    texs = {}
    for s in p.samplers:
        arr = targets[s.source] if isinstance(s.source, str) else s.source
        texs[s.field] = Tex((arr, s.filter, s.wrap, s.texel_div))
    sh = Shader(p.desc.shader, p.uniforms, p.layout, texs)
    pix = targets[p.pixel] if p.pixel else None
    dep = targets[p.depth] if p.depth else None
    pfmt = frame.target(p.pixel).fmt if p.pixel else abi.FMT_NONE
    return render(p.desc, sh, p.vertices, p.nverts, p.layout.stride, p.indices, pix, pfmt, dep)


def run_frame(frame):
    targets = frame.alloc_host_targets()
    res = [run_pass(frame, p, targets) for p in frame.passes]
    return targets, res
