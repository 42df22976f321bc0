"""FP64 central-difference gradients of the single-view L1 loss with the
forward's discrete decisions held (test infrastructure).

The loss is mean |out - target| over pixels and channels of the antialiased
interpolated image.  Its analytic gradient -- the one the reference gets from
dr.antialias (diffrp/rendering/surface_deferred.py:775) and the interpolation
autograd (diffrp/rendering/interpolator.py:32-48) -- is the gradient of the
image with every discrete decision of the forward fixed: each pixel's
triangle, each antialias pair's front triangle, crossing edge, blended pixel
and clamping, and the sign of out - target.  ``FixedVisibilityL1`` evaluates
that function in float64 through the oracle (orc_l1_fixed_visibility), so
its central differences check the backward without the discontinuities of
coverage changes: no pixel is excluded.

Step size.  Differences start at eps = 1e-3 and are refined by Ridders'
extrapolation (steps 1e-3 / 2^i, Neville tableau, the estimate with the
smallest change from its neighbours).  A single step of 1e-3 is not accurate
enough on its own at 1024 x 1024: one clip unit is about 160 pixels there,
and an antialias crossing parameter t = eF / (eF - eO) whose edge runs almost
parallel to the pixel step is a ratio of two small numbers, so a 0.16-pixel
step moves it far outside its linear range (the single-step error is
returned beside the extrapolated value for the record).
"""
import numpy as np

import oracle as O


class FixedVisibilityL1:
    def __init__(self, pos, tri, attr, target, rast, out, nbr=None):
        """pos (V, 4) float32 clip positions, tri (F, 3), attr (V, C),
        target / out (H, W, C) float32 (out: the forward's antialiased image),
        rast (H, W, 4) the forward's raster buffer."""
        rast = np.asarray(rast, np.float32).reshape(-1, 4)
        self.H, self.W, self.C = out.shape[-3], out.shape[-2], out.shape[-1]
        self.n = out.size
        self.tri = np.ascontiguousarray(tri, np.int32)
        self.pos = np.asarray(pos, np.float64)
        self.attr = np.asarray(attr, np.float64)
        r3 = rast[:, 3]
        # ids below 2^24 are exact float values (the encoding of interpolator.py:24-29)
        assert self.tri.shape[0] < (1 << 24)
        self.ids = np.where(r3 > 0, r3.astype(np.int64) - 1, -1).astype(np.int32)
        self.sign = np.sign(np.asarray(out, np.float32).reshape(-1) - np.asarray(target, np.float32).reshape(-1))
        self.sign = self.sign.astype(np.int8)
        self.plan = O.aa_plan(rast.reshape(self.H, self.W, 4), pos, self.tri, nbr)
        self.vert_tris = [[] for _ in range(self.pos.shape[0])]
        for t, tr in enumerate(self.tri):
            for k in tr:
                self.vert_tris[int(k)].append(t)

    def loss_terms(self, pos=None, attr=None, tri_flag=None):
        """Sum of sign * out (float64) over the terms touching flagged triangles."""
        return O.l1_fixed_visibility(self.pos if pos is None else pos, self.tri,
                                     self.attr if attr is None else attr, self.ids, self.sign, self.plan,
                                     (self.H, self.W), tri_flag)

    def _flag(self, vertex):
        flag = np.zeros(self.tri.shape[0], np.uint8)
        flag[self.vert_tris[vertex]] = 1
        return flag

    def _central(self, fn, eps):
        return (fn(eps) - fn(-eps)) / (2.0 * eps) / self.n

    def _ridders(self, fn, eps0=1e-3, levels=10):
        """Ridders' extrapolation of central differences from step eps0
        (steps eps0 / 2^i, every level evaluated: near a pole of the
        crossing parameter the first levels are far off, so the tableau is
        not cut short when an early level looks worse)."""
        fac0 = 4.0
        a = np.zeros((levels, levels))
        h = eps0
        a[0, 0] = self._central(fn, h)
        first = a[0, 0]
        best, err = a[0, 0], np.inf
        for i in range(1, levels):
            h /= 2.0
            a[0, i] = self._central(fn, h)
            fac = fac0
            for j in range(1, i + 1):
                a[j, i] = (a[j - 1, i] * fac - a[j - 1, i - 1]) / (fac - 1.0)
                fac *= fac0
                e = max(abs(a[j, i] - a[j - 1, i]), abs(a[j, i] - a[j - 1, i - 1]))
                if e <= err:
                    err, best = e, a[j, i]
        return best, first

    def grad_pos(self, vertex, coords=(0, 1, 2, 3), mvp=None, verts=None):
        """d mean-L1 / d position of one vertex: clip coordinates, or, with mvp
        (4 x 4) and verts (V, 3), world coordinates through clip = [v, 1] mvp^T
        in float64.  Returns (extrapolated, single step 1e-3)."""
        flag = self._flag(vertex)
        out, first = np.zeros(len(coords)), np.zeros(len(coords))
        for i, c in enumerate(coords):
            if mvp is None:
                def fn(e, c=c):
                    p = self.pos.copy()
                    p[vertex, c] += e
                    return self.loss_terms(pos=p, tri_flag=flag)
            else:
                M = np.asarray(mvp, np.float64)
                base = np.asarray(verts, np.float64)

                def fn(e, c=c):
                    v = base[vertex].copy()
                    v[c] += e
                    p = self.pos.copy()
                    p[vertex] = M[:, :3] @ v + M[:, 3]
                    return self.loss_terms(pos=p, tri_flag=flag)
            out[i], first[i] = self._ridders(fn)
        return out, first

    def grad_attr(self, vertex, eps=1e-3):
        """d mean-L1 / d attributes of one vertex (the loss is linear in them
        with the decisions held, so one central step is exact up to rounding)."""
        flag = self._flag(vertex)
        g = np.zeros(self.C)
        for c in range(self.C):
            def fn(e, c=c):
                a = self.attr.copy()
                a[vertex, c] += e
                return self.loss_terms(attr=a, tri_flag=flag)
            g[c] = self._central(fn, eps)
        return g

    def pick_vertices(self, count=64, seed=2024):
        """count seeded vertices: half among the vertices of visible
        triangles, half among those of antialias front triangles."""
        rng = np.random.default_rng(seed)
        vis = np.unique(self.tri[np.unique(self.ids[self.ids >= 0])].ravel())
        sil = np.unique(self.tri[np.unique(self.plan[:, 4])].ravel()) if len(self.plan) else vis
        a = rng.choice(vis, count // 2, replace=False)
        b = rng.choice(np.setdiff1d(sil, a), count - count // 2, replace=False)
        return np.concatenate([a, b])
