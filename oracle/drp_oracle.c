/*
 * drp_oracle.c -- CPU oracle for diffrp's rasterize -> interpolate -> antialias
 * hot path (forward and backward).
 *
 * TEST INFRASTRUCTURE ONLY.  tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg load this library as the checker (or as the timed CPU
 * baseline).  The product package never links, loads or calls it.
 *
 * What it restates
 * ----------------
 * Above the nvdiffrast boundary the arithmetic follows the reference's own code:
 *   - tri-id float encoding:       diffrp/rendering/interpolator.py:24-29
 *   - barycentric interpolation:   diffrp/rendering/interpolator.py:32-48
 *       result = fma(v1 - v3, u, fma(v2 - v3, v, v3))
 *   - rast channel meaning (u, v, z/w, tri_id + 1) and the barycentric
 *     convention u*v1 + v*v2 + (1-u-v)*v3 = p:
 *                                  diffrp/rendering/surface_deferred.py:240-266
 *   - antialias call contract:     diffrp/rendering/surface_deferred.py:758-775
 * Below the boundary (dr.rasterize / dr.interpolate / dr.antialias) the
 * reference delegates to the third-party package diffrp-nvdiffrast (setup.py:39,
 * unpinned, not present anywhere in the reference tree).  Its documented
 * semantics are restated from the mathematics:
 *   - pixel centres at half-integers, row 0 = NDC y = -1 (OpenGL, bottom-up);
 *   - visibility: nearest z/w in [-1, 1] wins; perspective-correct barycentrics
 *     solved in 2D homogeneous coordinates (Olano & Greer 1997);
 *   - rast_db = (du/dX, du/dY, dv/dX, dv/dY) in pixel units;
 *   - antialias: analytic silhouette-edge coverage blend between 4-neighbour
 *     pixel pairs (Laine et al. 2020, "Modular Primitives for High-Performance
 *     Differentiable Rendering", section on analytic antialiasing).
 * Snapping and fill-rule constants are this project's own (8 sub-pixel bits,
 * top-left rule in the y-up frame, guard band 64 NDC units) and are shared with
 * the CUDA kernels by specification, not by code.  Parity against nvdiffrast
 * itself is UNPINNED: no nvdiffrast source, binary or golden output exists in
 * the reference.
 *
 * Floating-point contract: compile with -ffp-contract=off.  Every float
 * expression is evaluated in the written order with one rounding per operation;
 * fused multiply-adds appear only as explicit fmaf()/fma() calls.  The CUDA
 * kernels are compiled with --fmad=false and follow the same operation order,
 * which makes visibility, rast and the forward images bit-identical.
 *
 * REAL selects the shading precision: float (bit-exact parity build) or double
 * (finite-difference and gradient reference build).  Coverage always snaps in
 * float so both builds agree on visibility.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef REAL
#define REAL float
#endif
typedef REAL real;

#define SUBPIX_BITS 8
#define SUBPIX 256
#define HALF_SUBPIX 128
#define GUARD 64.0f
#define MAX_POLY 8

#define ORC_OK 0
#define ORC_MAX_AA_CHANNELS 256
#define ORC_BAD_INDEX 3

#if defined(__GNUC__)
#define ORC_EXPORT __attribute__((visibility("default")))
#else
#define ORC_EXPORT
#endif

static inline real r_fma(real a, real b, real c) {
#ifdef REAL_IS_DOUBLE
    return fma(a, b, c);
#else
    return fmaf(a, b, c);
#endif
}

/* ---------------------------------------------------------------------- */
/* tri-id encoding (interpolator.py:24-29)                                  */
/* ---------------------------------------------------------------------- */
static inline float enc_triid(int32_t id1) {
    if (id1 <= 0x01000000) return (float)id1;
    uint32_t b = 0x4a800000u + (uint32_t)id1;
    float f;
    memcpy(&f, &b, 4);
    return f;
}

static inline int32_t dec_triid(float f) {
    if (f <= 16777216.0f) return (int32_t)f;
    uint32_t b;
    memcpy(&b, &f, 4);
    return (int32_t)(b - 0x4a800000u);
}

ORC_EXPORT float orc_triidx_to_float(int32_t id1) { return enc_triid(id1); }
ORC_EXPORT int32_t orc_float_to_triidx(float f) { return dec_triid(f); }

static inline uint32_t depth_order(float z) {
    uint32_t b;
    memcpy(&b, &z, 4);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

static inline int64_t floor_shift(int64_t a) { return a >> SUBPIX_BITS; }
static inline int64_t ceil_shift(int64_t a) { return -((-a) >> SUBPIX_BITS); }

/* ---------------------------------------------------------------------- */
/* Triangle setup: trivial reject, near/guard clipping, projection, snap.   */
/* ---------------------------------------------------------------------- */
typedef struct {
    int n;                 /* polygon vertices after clipping (0 = culled) */
    int32_t X[MAX_POLY];   /* fixed-point screen x (1/256 px) */
    int32_t Y[MAX_POLY];
    float Z[MAX_POLY];     /* z/w */
} poly_t;

static inline float plane_dist(const float* p, int plane) {
    switch (plane) {
    case 0: return p[2] + p[3];          /* near: z >= -w */
    case 1: return GUARD * p[3] - p[0];  /* x <= G w */
    case 2: return p[0] + GUARD * p[3];  /* x >= -G w */
    case 3: return GUARD * p[3] - p[1];  /* y <= G w */
    default: return p[1] + GUARD * p[3]; /* y >= -G w */
    }
}

/* Half-space tests for trivial reject: view frustum planes in clip space. */
static inline float frustum_dist(const float* p, int plane) {
    switch (plane) {
    case 0: return p[3] + p[0];  /* x >= -w */
    case 1: return p[3] - p[0];  /* x <= w */
    case 2: return p[3] + p[1];  /* y >= -w */
    case 3: return p[3] - p[1];  /* y <= w */
    case 4: return p[3] + p[2];  /* z >= -w */
    default: return p[3] - p[2]; /* z <= w */
    }
}

static int clip_polygon(float (*poly)[4], int n, int plane, float (*out)[4]) {
    int m = 0;
    for (int i = 0; i < n; ++i) {
        const float* p = poly[i];
        const float* q = poly[(i + 1) % n];
        float dp = plane_dist(p, plane);
        float dq = plane_dist(q, plane);
        int pin = dp >= 0.0f, qin = dq >= 0.0f;
        if (pin) {
            memcpy(out[m], p, sizeof(float) * 4);
            ++m;
        }
        if (pin != qin) {
            float t = dp / (dp - dq);
            for (int c = 0; c < 4; ++c) out[m][c] = p[c] + t * (q[c] - p[c]);
            ++m;
        }
    }
    return m;
}

static inline int32_t snap_coord(float c, float w, int res) {
    float q = c / w;
    float s = (q + 1.0f) * (float)(res * HALF_SUBPIX);
    return (int32_t)nearbyintf(s);
}

static void setup_triangle(const float* p0, const float* p1, const float* p2, int W, int H, poly_t* out) {
    out->n = 0;
    const float* v[3] = {p0, p1, p2};
    for (int i = 0; i < 3; ++i)
        for (int c = 0; c < 4; ++c)
            if (!isfinite(v[i][c])) return;
    for (int pl = 0; pl < 6; ++pl) {
        if (frustum_dist(p0, pl) < 0.0f && frustum_dist(p1, pl) < 0.0f && frustum_dist(p2, pl) < 0.0f) return;
    }
    float poly[MAX_POLY][4], tmp[MAX_POLY][4];
    int n = 3;
    for (int i = 0; i < 3; ++i) memcpy(poly[i], v[i], sizeof(float) * 4);
    int need = 0;
    for (int i = 0; i < 3; ++i) {
        if (!(v[i][3] > 0.0f)) need = 1;
        for (int pl = 0; pl < 5; ++pl)
            if (plane_dist(v[i], pl) < 0.0f) need = 1;
    }
    if (need) {
        for (int pl = 0; pl < 5 && n >= 3; ++pl) {
            n = clip_polygon(poly, n, pl, tmp);
            memcpy(poly, tmp, sizeof(float) * 4 * (size_t)n);
        }
        if (n < 3) return;
        for (int i = 0; i < n; ++i)
            if (!(poly[i][3] > 0.0f)) return;
    }
    for (int i = 0; i < n; ++i) {
        out->X[i] = snap_coord(poly[i][0], poly[i][3], W);
        out->Y[i] = snap_coord(poly[i][1], poly[i][3], H);
        out->Z[i] = poly[i][2] / poly[i][3];
    }
    out->n = n;
}

/* Edge inclusion with the top-left rule (y-up frame, CCW orientation). */
static inline int edge_inside(int64_t ax, int64_t ay, int64_t bx, int64_t by, int64_t cx, int64_t cy) {
    int64_t dx = bx - ax, dy = by - ay;
    int64_t e = dx * (cy - ay) - dy * (cx - ax);
    if (e > 0) return 1;
    if (e < 0) return 0;
    return (dy < 0) || (dy == 0 && dx < 0);
}

/* Rasterise one fan sub-triangle of a setup polygon into key[] rows [y0, y1). */
static void raster_subtri(int64_t X0, int64_t Y0, float Z0, int64_t X1, int64_t Y1, float Z1,
                          int64_t X2, int64_t Y2, float Z2, uint32_t tri, int W, int y0, int y1,
                          const uint64_t* prev, uint64_t* key) {
    int64_t area2 = (X1 - X0) * (Y2 - Y0) - (Y1 - Y0) * (X2 - X0);
    if (area2 == 0) return;
    /* depth plane z = Z0 + A (cx - X0) + B (cy - Y0), fan order, before any swap */
    float dx1 = (float)(X1 - X0), dy1 = (float)(Y1 - Y0);
    float dx2 = (float)(X2 - X0), dy2 = (float)(Y2 - Y0);
    float dz1 = Z1 - Z0, dz2 = Z2 - Z0;
    float det = (float)area2;
    float A = (dz1 * dy2 - dy1 * dz2) / det;
    float B = (dx1 * dz2 - dz1 * dx2) / det;
    int64_t ax = X0, ay = Y0, bx = X1, by = Y1, cx = X2, cy = Y2;
    if (area2 < 0) { bx = X2; by = Y2; cx = X1; cy = Y1; }
    int64_t mnx = X0 < X1 ? X0 : X1; mnx = mnx < X2 ? mnx : X2;
    int64_t mxx = X0 > X1 ? X0 : X1; mxx = mxx > X2 ? mxx : X2;
    int64_t mny = Y0 < Y1 ? Y0 : Y1; mny = mny < Y2 ? mny : Y2;
    int64_t mxy = Y0 > Y1 ? Y0 : Y1; mxy = mxy > Y2 ? mxy : Y2;
    int64_t px0 = ceil_shift(mnx - HALF_SUBPIX), px1 = floor_shift(mxx - HALF_SUBPIX);
    int64_t py0 = ceil_shift(mny - HALF_SUBPIX), py1 = floor_shift(mxy - HALF_SUBPIX);
    if (px0 < 0) px0 = 0;
    if (px1 > W - 1) px1 = W - 1;
    if (py0 < y0) py0 = y0;
    if (py1 > y1 - 1) py1 = y1 - 1;
    for (int64_t py = py0; py <= py1; ++py) {
        int64_t sy = py * SUBPIX + HALF_SUBPIX;
        for (int64_t px = px0; px <= px1; ++px) {
            int64_t sx = px * SUBPIX + HALF_SUBPIX;
            if (!edge_inside(bx, by, cx, cy, sx, sy)) continue;
            if (!edge_inside(cx, cy, ax, ay, sx, sy)) continue;
            if (!edge_inside(ax, ay, bx, by, sx, sy)) continue;
            float z = (Z0 + A * (float)(sx - X0)) + B * (float)(sy - Y0);
            if (!(z >= -1.0f && z <= 1.0f)) continue;
            uint64_t k = ((uint64_t)depth_order(z) << 32) | (uint64_t)tri;
            size_t pix = (size_t)py * (size_t)W + (size_t)px;
            if (prev && !(k > prev[pix])) continue;
            if (k < key[pix]) key[pix] = k;
        }
    }
}

#define BAND 32

/*
 * Visibility: per pixel 64-bit key = (ordered z/w << 32) | triangle index.
 * The minimum key wins, which makes exact depth ties resolve to the lower
 * triangle index.  With prev_key, only keys strictly greater than the previous
 * layer's key are eligible (depth peeling).  Background = UINT64_MAX.
 */
ORC_EXPORT int orc_raster_ids(const float* pos, long pos_view_stride, long V, const int32_t* tri, long F,
                              const int32_t* tri_first, const int32_t* tri_count, int B, int H, int W,
                              const uint64_t* prev_key, uint64_t* out_key, int nthreads) {
    for (int b = 0; b < B; ++b) {
        if (tri_first[b] < 0 || tri_count[b] < 0 || (long)tri_first[b] + tri_count[b] > F) return ORC_BAD_INDEX;
        for (long t = tri_first[b]; t < (long)tri_first[b] + tri_count[b]; ++t)
            for (int k = 0; k < 3; ++k)
                if (tri[t * 3 + k] < 0 || tri[t * 3 + k] >= V) return ORC_BAD_INDEX;
    }
    size_t npix = (size_t)H * (size_t)W;
    for (size_t i = 0; i < npix * (size_t)B; ++i) out_key[i] = UINT64_MAX;
    int nbands = (H + BAND - 1) / BAND;
    long njobs = (long)B * nbands;
    (void)nthreads;
#pragma omp parallel for schedule(dynamic) num_threads(nthreads > 0 ? nthreads : 1)
    for (long job = 0; job < njobs; ++job) {
        int b = (int)(job / nbands), band = (int)(job % nbands);
        int y0 = band * BAND, y1 = y0 + BAND < H ? y0 + BAND : H;
        const float* P = pos + (size_t)b * (size_t)pos_view_stride;
        uint64_t* key = out_key + (size_t)b * npix;
        const uint64_t* prev = prev_key ? prev_key + (size_t)b * npix : NULL;
        for (long t = tri_first[b]; t < (long)tri_first[b] + tri_count[b]; ++t) {
            const int32_t* ti = tri + t * 3;
            poly_t poly;
            setup_triangle(P + (size_t)ti[0] * 4, P + (size_t)ti[1] * 4, P + (size_t)ti[2] * 4, W, H, &poly);
            for (int i = 1; i + 1 < poly.n; ++i)
                raster_subtri(poly.X[0], poly.Y[0], poly.Z[0], poly.X[i], poly.Y[i], poly.Z[i], poly.X[i + 1],
                              poly.Y[i + 1], poly.Z[i + 1], (uint32_t)t, W, y0, y1, prev, key);
        }
    }
    return ORC_OK;
}

/* ---------------------------------------------------------------------- */
/* Perspective-correct barycentrics, z/w and their screen derivatives.      */
/* ---------------------------------------------------------------------- */
typedef struct {
    real a[3], c[3], n[3], s;
    real u, v, nz, nw, zw;
    real Dx[3], Dy[3], Sx, Sy;
    real X, Y, kx, ky;
} shade_t;

static void shade_eval(const real* p0, const real* p1, const real* p2, int px, int py, int W, int H, shade_t* S) {
    const real* p[3] = {p0, p1, p2};
    S->X = (real)(2 * px + 1) / (real)W - (real)1;
    S->Y = (real)(2 * py + 1) / (real)H - (real)1;
    for (int i = 0; i < 3; ++i) {
        S->a[i] = p[i][0] - S->X * p[i][3];
        S->c[i] = p[i][1] - S->Y * p[i][3];
    }
    real *a = S->a, *c = S->c;
    S->n[0] = a[1] * c[2] - a[2] * c[1];
    S->n[1] = a[2] * c[0] - a[0] * c[2];
    S->n[2] = a[0] * c[1] - a[1] * c[0];
    S->s = (S->n[0] + S->n[1]) + S->n[2];
    S->u = S->n[0] / S->s;
    S->v = S->n[1] / S->s;
    S->nz = (S->n[0] * p0[2] + S->n[1] * p1[2]) + S->n[2] * p2[2];
    S->nw = (S->n[0] * p0[3] + S->n[1] * p1[3]) + S->n[2] * p2[3];
    S->zw = S->nz / S->nw;
    real w0 = p0[3], w1 = p1[3], w2 = p2[3];
    S->Dx[0] = c[1] * w2 - c[2] * w1;
    S->Dx[1] = c[2] * w0 - c[0] * w2;
    S->Dx[2] = c[0] * w1 - c[1] * w0;
    S->Dy[0] = w1 * a[2] - w2 * a[1];
    S->Dy[1] = w2 * a[0] - w0 * a[2];
    S->Dy[2] = w0 * a[1] - w1 * a[0];
    S->Sx = (S->Dx[0] + S->Dx[1]) + S->Dx[2];
    S->Sy = (S->Dy[0] + S->Dy[1]) + S->Dy[2];
    S->kx = (real)2 / (real)W;
    S->ky = (real)2 / (real)H;
}

static inline int32_t key_tri(uint64_t k) { return k == UINT64_MAX ? -1 : (int32_t)(uint32_t)(k & 0xffffffffu); }

ORC_EXPORT int orc_shade(const real* pos, long pos_view_stride, long V, const int32_t* tri, long F,
                         const uint64_t* key, int B, int H, int W, real* rast, real* rast_db, int nthreads) {
    (void)V; (void)F; (void)nthreads;
    long npix = (long)H * W;
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
    for (long i = 0; i < (long)B * npix; ++i) {
        int b = (int)(i / npix);
        long pix = i % npix;
        int py = (int)(pix / W), px = (int)(pix % W);
        int32_t t = key_tri(key[i]);
        real* r = rast + i * 4;
        real* d = rast_db ? rast_db + i * 4 : NULL;
        if (t < 0) {
            r[0] = r[1] = r[2] = r[3] = 0;
            if (d) d[0] = d[1] = d[2] = d[3] = 0;
            continue;
        }
        const real* P = pos + (size_t)b * (size_t)pos_view_stride;
        const int32_t* ti = tri + (size_t)t * 3;
        shade_t S;
        shade_eval(P + (size_t)ti[0] * 4, P + (size_t)ti[1] * 4, P + (size_t)ti[2] * 4, px, py, W, H, &S);
        r[0] = S.u;
        r[1] = S.v;
        r[2] = S.zw;
        r[3] = (real)enc_triid(t + 1);
        if (d) {
            d[0] = ((S.Dx[0] - S.u * S.Sx) / S.s) * S.kx;
            d[1] = ((S.Dy[0] - S.u * S.Sy) / S.s) * S.ky;
            d[2] = ((S.Dx[1] - S.v * S.Sx) / S.s) * S.kx;
            d[3] = ((S.Dy[1] - S.v * S.Sy) / S.s) * S.ky;
        }
    }
    return ORC_OK;
}

static inline void cross3(const real* x, const real* y, real* o) {
    o[0] = x[1] * y[2] - x[2] * y[1];
    o[1] = x[2] * y[0] - x[0] * y[2];
    o[2] = x[0] * y[1] - x[1] * y[0];
}

/*
 * Gradient of (u, v, z/w) and of rast_db w.r.t. the three clip-space vertices.
 * g = dL/d(u, v, z/w); gdb = dL/d(du/dX, du/dY, dv/dX, dv/dY) or NULL.
 * out[i*4 + c] receives dL/d(p_i.c).
 */
static void shade_grad(const real* p0, const real* p1, const real* p2, const shade_t* S, const real* g,
                       const real* gdb, double* out) {
    const real* p[3] = {p0, p1, p2};
    real b[3] = {S->u, S->v, S->n[2] / S->s};
    real gb[3] = {g[0], g[1], 0};
    real beta = gb[0] * b[0] + gb[1] * b[1];
    real gn[3], gzc[3], gwd[3];
    real d = S->zw;
    for (int i = 0; i < 3; ++i) {
        gn[i] = (gb[i] - beta) / S->s + g[2] * (p[i][2] - d * p[i][3]) / S->nw;
        gzc[i] = g[2] * S->n[i] / S->nw;
        gwd[i] = -g[2] * d * S->n[i] / S->nw;
    }
    real qX[3] = {0, 0, 0}, qY[3] = {0, 0, 0};
    if (gdb) {
        real GX[3] = {gdb[0] * S->kx, gdb[2] * S->kx, 0};
        real GY[3] = {gdb[1] * S->ky, gdb[3] * S->ky, 0};
        real gamX = GX[0] * b[0] + GX[1] * b[1];
        real gamY = GY[0] * b[0] + GY[1] * b[1];
        real LX = 0, LY = 0;
        for (int i = 0; i < 2; ++i) {
            LX += GX[i] * (S->Dx[i] - b[i] * S->Sx) / S->s;
            LY += GY[i] * (S->Dy[i] - b[i] * S->Sy) / S->s;
        }
        for (int j = 0; j < 3; ++j) {
            qX[j] = (GX[j] - gamX) / S->s;
            qY[j] = (GY[j] - gamY) / S->s;
            gn[j] += -(S->Sx / S->s) * qX[j] - LX / S->s;
            gn[j] += -(S->Sy / S->s) * qY[j] - LY / S->s;
        }
    }
    /* n = a x c, Dx = c x w, Dy = w x a */
    real wv[3] = {p0[3], p1[3], p2[3]};
    real t1[3], t2[3], ga[3], gc[3], gw[3];
    cross3(S->c, gn, t1);
    cross3(qY, wv, t2);
    for (int i = 0; i < 3; ++i) ga[i] = t1[i] + t2[i];
    cross3(gn, S->a, t1);
    cross3(wv, qX, t2);
    for (int i = 0; i < 3; ++i) gc[i] = t1[i] + t2[i];
    cross3(qX, S->c, t1);
    cross3(S->a, qY, t2);
    for (int i = 0; i < 3; ++i) gw[i] = t1[i] + t2[i];
    for (int i = 0; i < 3; ++i) {
        out[i * 4 + 0] += ga[i];
        out[i * 4 + 1] += gc[i];
        out[i * 4 + 2] += gzc[i];
        out[i * 4 + 3] += -S->X * ga[i] - S->Y * gc[i] + gw[i] + gwd[i];
    }
}

static inline int32_t rast_tri(const real* r) {
    float f = (float)r[3];
    if (!(f > 0.0f)) return -1;
    return dec_triid(f) - 1;
}

static int max_threads(int nthreads) { return nthreads > 0 ? nthreads : 1; }

/* grad_pos: accumulated (+=), same layout as pos (views x V x 4 or V x 4). */
ORC_EXPORT int orc_raster_bwd(const real* pos, long pos_view_stride, long V, const int32_t* tri, long F,
                              const real* rast, const real* grad_rast, const real* grad_db, int B, int H, int W,
                              double* grad_pos, int nthreads) {
    (void)F;
    long npix = (long)H * W;
    int nt = max_threads(nthreads);
    long gsize = (pos_view_stride ? (long)B : 1) * V * 4;
    double* acc = (double*)calloc((size_t)nt * (size_t)gsize, sizeof(double));
    if (!acc) return 1;
#pragma omp parallel num_threads(nt)
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        double* A = acc + (size_t)tid * (size_t)gsize;
#pragma omp for schedule(static)
        for (long i = 0; i < (long)B * npix; ++i) {
            int32_t t = rast_tri(rast + i * 4);
            if (t < 0) continue;
            int b = (int)(i / npix);
            long pix = i % npix;
            int py = (int)(pix / W), px = (int)(pix % W);
            const real* P = pos + (size_t)b * (size_t)pos_view_stride;
            const int32_t* ti = tri + (size_t)t * 3;
            shade_t S;
            shade_eval(P + (size_t)ti[0] * 4, P + (size_t)ti[1] * 4, P + (size_t)ti[2] * 4, px, py, W, H, &S);
            double out[12] = {0};
            shade_grad(P + (size_t)ti[0] * 4, P + (size_t)ti[1] * 4, P + (size_t)ti[2] * 4, &S, grad_rast + i * 4,
                       grad_db ? grad_db + i * 4 : NULL, out);
            double* G = A + (pos_view_stride ? (size_t)b * (size_t)V * 4 : 0);
            for (int k = 0; k < 3; ++k)
                for (int c = 0; c < 4; ++c) G[(size_t)ti[k] * 4 + c] += out[k * 4 + c];
        }
    }
    for (int th = 0; th < nt; ++th)
        for (long j = 0; j < gsize; ++j) grad_pos[j] += acc[(size_t)th * (size_t)gsize + j];
    free(acc);
    return ORC_OK;
}

/* ---------------------------------------------------------------------- */
/* Interpolation (interpolator.py:32-48 order of operations).               */
/* ---------------------------------------------------------------------- */
ORC_EXPORT int orc_interp_fwd(const real* attr, long attr_view_stride, long V, int C, const real* rast,
                              const real* rast_db, const int32_t* tri, long F, int B, int H, int W,
                              const int32_t* diff_idx, int nd, real* out, real* da, int nthreads) {
    (void)V; (void)F;
    long npix = (long)H * W;
#pragma omp parallel for schedule(static) num_threads(max_threads(nthreads))
    for (long i = 0; i < (long)B * npix; ++i) {
        int b = (int)(i / npix);
        real* o = out + i * C;
        real* dd = da ? da + i * 2 * nd : NULL;
        int32_t t = rast_tri(rast + i * 4);
        if (t < 0) {
            for (int c = 0; c < C; ++c) o[c] = 0;
            if (dd) for (int c = 0; c < 2 * nd; ++c) dd[c] = 0;
            continue;
        }
        const real* Aa = attr + (size_t)b * (size_t)attr_view_stride;
        const int32_t* ti = tri + (size_t)t * 3;
        const real *a0 = Aa + (size_t)ti[0] * C, *a1 = Aa + (size_t)ti[1] * C, *a2 = Aa + (size_t)ti[2] * C;
        real u = rast[i * 4 + 0], v = rast[i * 4 + 1];
        for (int c = 0; c < C; ++c) o[c] = r_fma(a0[c] - a2[c], u, r_fma(a1[c] - a2[c], v, a2[c]));
        if (dd) {
            const real* db = rast_db + i * 4;
            for (int k = 0; k < nd; ++k) {
                int c = diff_idx[k];
                real e0 = a0[c] - a2[c], e1 = a1[c] - a2[c];
                dd[2 * k + 0] = r_fma(e0, db[0], e1 * db[2]);
                dd[2 * k + 1] = r_fma(e0, db[1], e1 * db[3]);
            }
        }
    }
    return ORC_OK;
}

/* grad_attr accumulated (+=) in double; grad_rast / grad_db overwritten (channels 2,3 zero). */
ORC_EXPORT int orc_interp_bwd(const real* attr, long attr_view_stride, long V, int C, const real* rast,
                              const real* rast_db, const int32_t* tri, long F, int B, int H, int W,
                              const int32_t* diff_idx, int nd, const real* grad_out, const real* grad_da,
                              double* grad_attr, real* grad_rast, real* grad_db, int nthreads) {
    (void)F;
    long npix = (long)H * W;
    int nt = max_threads(nthreads);
    long gsize = (attr_view_stride ? (long)B : 1) * V * C;
    double* acc = (double*)calloc((size_t)nt * (size_t)gsize, sizeof(double));
    if (!acc) return 1;
#pragma omp parallel num_threads(nt)
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        double* A = acc + (size_t)tid * (size_t)gsize;
#pragma omp for schedule(static)
        for (long i = 0; i < (long)B * npix; ++i) {
            int b = (int)(i / npix);
            real* gr = grad_rast + i * 4;
            gr[0] = gr[1] = gr[2] = gr[3] = 0;
            real* gd = grad_db ? grad_db + i * 4 : NULL;
            if (gd) gd[0] = gd[1] = gd[2] = gd[3] = 0;
            int32_t t = rast_tri(rast + i * 4);
            if (t < 0) continue;
            const real* Aa = attr + (size_t)b * (size_t)attr_view_stride;
            double* G = A + (attr_view_stride ? (size_t)b * (size_t)V * C : 0);
            const int32_t* ti = tri + (size_t)t * 3;
            const real *a0 = Aa + (size_t)ti[0] * C, *a1 = Aa + (size_t)ti[1] * C, *a2 = Aa + (size_t)ti[2] * C;
            real u = rast[i * 4 + 0], v = rast[i * 4 + 1], w = (real)1 - u - v;
            const real* g = grad_out + i * C;
            double gu = 0, gv = 0;
            for (int c = 0; c < C; ++c) {
                G[(size_t)ti[0] * C + c] += (double)g[c] * u;
                G[(size_t)ti[1] * C + c] += (double)g[c] * v;
                G[(size_t)ti[2] * C + c] += (double)g[c] * w;
                gu += (double)g[c] * (a0[c] - a2[c]);
                gv += (double)g[c] * (a1[c] - a2[c]);
            }
            gr[0] = (real)gu;
            gr[1] = (real)gv;
            if (grad_da && nd > 0) {
                const real* db = rast_db + i * 4;
                const real* gdd = grad_da + i * 2 * nd;
                double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
                for (int k = 0; k < nd; ++k) {
                    int c = diff_idx[k];
                    real gx = gdd[2 * k], gy = gdd[2 * k + 1];
                    real e0 = a0[c] - a2[c], e1 = a1[c] - a2[c];
                    double w0 = (double)gx * db[0] + (double)gy * db[1];
                    double w1 = (double)gx * db[2] + (double)gy * db[3];
                    G[(size_t)ti[0] * C + c] += w0;
                    G[(size_t)ti[1] * C + c] += w1;
                    G[(size_t)ti[2] * C + c] -= w0 + w1;
                    s0 += (double)gx * e0;
                    s1 += (double)gy * e0;
                    s2 += (double)gx * e1;
                    s3 += (double)gy * e1;
                }
                if (gd) {
                    gd[0] = (real)s0;
                    gd[1] = (real)s1;
                    gd[2] = (real)s2;
                    gd[3] = (real)s3;
                }
            }
        }
    }
    for (int th = 0; th < nt; ++th)
        for (long j = 0; j < gsize; ++j) grad_attr[j] += acc[(size_t)th * (size_t)gsize + j];
    free(acc);
    return ORC_OK;
}

/* Sparse (stencil-masked) interpolation: interpolator.py:32-48 on (N, 4) vi_data. */
ORC_EXPORT int orc_interp_sparse_fwd(const real* vb, long V, int C, const real* vi, const int64_t* tri_idx, long N,
                                     real* out) {
    for (long n = 0; n < N; ++n) {
        const int64_t* ti = tri_idx + n * 3;
        for (int k = 0; k < 3; ++k)
            if (ti[k] < 0 || ti[k] >= V) return ORC_BAD_INDEX;
        const real *a0 = vb + ti[0] * C, *a1 = vb + ti[1] * C, *a2 = vb + ti[2] * C;
        real u = vi[n * 4 + 0], v = vi[n * 4 + 1];
        for (int c = 0; c < C; ++c) out[n * C + c] = r_fma(a0[c] - a2[c], u, r_fma(a1[c] - a2[c], v, a2[c]));
    }
    return ORC_OK;
}

/* ---------------------------------------------------------------------- */
/* Edge topology: for triangle t and edge k (vertices k+1, k+2 mod 3), the   */
/* other triangle sharing the unordered vertex pair when exactly two do.    */
/* ---------------------------------------------------------------------- */
typedef struct { uint64_t key; int32_t t, k; } edge_rec;

static int edge_cmp(const void* a, const void* b) {
    const edge_rec *x = (const edge_rec*)a, *y = (const edge_rec*)b;
    if (x->key != y->key) return x->key < y->key ? -1 : 1;
    if (x->t != y->t) return x->t < y->t ? -1 : 1;
    return x->k - y->k;
}

ORC_EXPORT int orc_topology(const int32_t* tri, long F, int32_t* nbr) {
    edge_rec* e = (edge_rec*)malloc(sizeof(edge_rec) * (size_t)(3 * F + 1));
    if (!e) return 1;
    for (long t = 0; t < F; ++t)
        for (int k = 0; k < 3; ++k) {
            uint32_t a = (uint32_t)tri[t * 3 + (k + 1) % 3], b = (uint32_t)tri[t * 3 + (k + 2) % 3];
            uint32_t lo = a < b ? a : b, hi = a < b ? b : a;
            e[t * 3 + k].key = ((uint64_t)lo << 32) | hi;
            e[t * 3 + k].t = (int32_t)t;
            e[t * 3 + k].k = k;
            nbr[t * 3 + k] = -1;
        }
    qsort(e, (size_t)(3 * F), sizeof(edge_rec), edge_cmp);
    long i = 0;
    while (i < 3 * F) {
        long j = i;
        while (j < 3 * F && e[j].key == e[i].key) ++j;
        if (j - i == 2 && e[i].t != e[i + 1].t && (e[i].key >> 32) != (e[i].key & 0xffffffffu)) {
            nbr[(long)e[i].t * 3 + e[i].k] = e[i + 1].t;
            nbr[(long)e[i + 1].t * 3 + e[i + 1].k] = e[i].t;
        }
        i = j;
    }
    free(e);
    return ORC_OK;
}

/* ---------------------------------------------------------------------- */
/* Analytic silhouette antialiasing.                                        */
/* ---------------------------------------------------------------------- */
typedef struct {
    int valid;
    long target, src;      /* pixel indices within the view */
    real w;                /* blend weight: out[target] += w (c[src] - c[target]) */
    real sign;             /* dw/dt */
    int32_t T;             /* front triangle */
    int k;                 /* crossing edge */
    real eF, eO, t;
    int clamped;
    real sgn;              /* orientation sign of T in screen space */
    real s[3][2];          /* projected vertices */
    real cF[2], cO[2];
} aa_pair_t;

static inline real edge_fn(const real* a, const real* b, const real* p) {
    return (b[0] - a[0]) * (p[1] - a[1]) - (b[1] - a[1]) * (p[0] - a[0]);
}

static int project_vertex(const real* p, int W, int H, real* s) {
    if (!(p[3] > 0)) return 0;
    s[0] = (p[0] / p[3] + (real)1) * ((real)W * (real)0.5);
    s[1] = (p[1] / p[3] + (real)1) * ((real)H * (real)0.5);
    return 1;
}

/*
 * Evaluate the unordered pixel pair (A, B) with B the right or upper neighbour
 * of A.  Both members of a pair reach the same decision, so the forward pass can
 * gather per pixel without atomics.
 */
static void aa_pair(const real* rast, const real* P, const int32_t* tri, const int32_t* nbr, int W, int H,
                    long A, long Bp, aa_pair_t* R) {
    R->valid = 0;
    int32_t tA = rast_tri(rast + A * 4), tB = rast_tri(rast + Bp * 4);
    if (tA == tB) return;
    long Fp, Op;
    if (tA < 0) Fp = Bp;
    else if (tB < 0) Fp = A;
    else {
        real zA = rast[A * 4 + 2], zB = rast[Bp * 4 + 2];
        if (zA < zB) Fp = A;
        else if (zB < zA) Fp = Bp;
        else Fp = tA < tB ? A : Bp;
    }
    Op = Fp == A ? Bp : A;
    int32_t T = Fp == A ? tA : tB;
    const int32_t* ti = tri + (size_t)T * 3;
    for (int i = 0; i < 3; ++i)
        if (!project_vertex(P + (size_t)ti[i] * 4, W, H, R->s[i])) return;
    real area = (R->s[1][0] - R->s[0][0]) * (R->s[2][1] - R->s[0][1]) -
                (R->s[1][1] - R->s[0][1]) * (R->s[2][0] - R->s[0][0]);
    if (area == 0 || area != area) return;
    real sgn = area > 0 ? (real)1 : (real)-1;
    R->cF[0] = (real)(Fp % W) + (real)0.5;
    R->cF[1] = (real)(Fp / W) + (real)0.5;
    R->cO[0] = (real)(Op % W) + (real)0.5;
    R->cO[1] = (real)(Op / W) + (real)0.5;
    int best = -1;
    real bt = 0, beF = 0, beO = 0;
    for (int k = 0; k < 3; ++k) {
        const real* a = R->s[(k + 1) % 3];
        const real* b = R->s[(k + 2) % 3];
        real eO = sgn * edge_fn(a, b, R->cO);
        if (!(eO < 0)) continue;
        real eF = sgn * edge_fn(a, b, R->cF);
        real t = eF / (eF - eO);
        if (best < 0 || t < bt) {
            best = k;
            bt = t;
            beF = eF;
            beO = eO;
        }
    }
    if (best < 0) return;
    int32_t N = nbr ? nbr[(size_t)T * 3 + best] : -1;
    if (N >= 0) {
        const int32_t* ni = tri + (size_t)N * 3;
        int32_t ea = ti[(best + 1) % 3], eb = ti[(best + 2) % 3];
        int32_t opp = -1;
        for (int i = 0; i < 3; ++i)
            if (ni[i] != ea && ni[i] != eb) opp = ni[i];
        real so[2];
        if (opp >= 0 && project_vertex(P + (size_t)opp * 4, W, H, so)) {
            const real* a = R->s[(best + 1) % 3];
            const real* b = R->s[(best + 2) % 3];
            real dT = edge_fn(a, b, R->s[best]);
            real dN = edge_fn(a, b, so);
            if ((dT > 0 && dN < 0) || (dT < 0 && dN > 0)) return; /* interior edge */
        }
    }
    R->clamped = 0;
    if (bt < 0) { bt = 0; R->clamped = 1; }
    if (bt > 1) { bt = 1; R->clamped = 1; }
    R->T = T;
    R->k = best;
    R->eF = beF;
    R->eO = beO;
    R->t = bt;
    R->sgn = sgn;
    if (bt > (real)0.5) {
        R->target = Op;
        R->src = Fp;
        R->w = bt - (real)0.5;
        R->sign = 1;
    } else {
        R->target = Fp;
        R->src = Op;
        R->w = (real)0.5 - bt;
        R->sign = -1;
    }
    R->valid = 1;
}

ORC_EXPORT int orc_aa_fwd(const real* color, int C, const real* rast, const real* pos, long pos_view_stride, long V,
                          const int32_t* tri, long F, const int32_t* nbr, int B, int H, int W, real* out,
                          int nthreads) {
    (void)V; (void)F;
    long npix = (long)H * W;
#pragma omp parallel for schedule(static) num_threads(max_threads(nthreads))
    for (long i = 0; i < (long)B * npix; ++i) {
        int b = (int)(i / npix);
        long pix = i % npix;
        int py = (int)(pix / W), px = (int)(pix % W);
        const real* R = rast + (size_t)b * (size_t)npix * 4;
        const real* Cc = color + (size_t)b * (size_t)npix * C;
        const real* P = pos + (size_t)b * (size_t)pos_view_stride;
        real* o = out + i * C;
        for (int c = 0; c < C; ++c) o[c] = Cc[pix * C + c];
        long pairs[4][2];
        int np = 0;
        if (px > 0) { pairs[np][0] = pix - 1; pairs[np][1] = pix; ++np; }
        if (px < W - 1) { pairs[np][0] = pix; pairs[np][1] = pix + 1; ++np; }
        if (py > 0) { pairs[np][0] = pix - W; pairs[np][1] = pix; ++np; }
        if (py < H - 1) { pairs[np][0] = pix; pairs[np][1] = pix + W; ++np; }
        for (int q = 0; q < np; ++q) {
            aa_pair_t pr;
            aa_pair(R, P, tri, nbr, W, H, pairs[q][0], pairs[q][1], &pr);
            if (!pr.valid || pr.target != pix) continue;
            for (int c = 0; c < C; ++c) o[c] = r_fma(pr.w, Cc[pr.src * C + c] - Cc[pix * C + c], o[c]);
        }
    }
    return ORC_OK;
}

/* grad_color overwritten; grad_pos accumulated (+=) in double. */
ORC_EXPORT int orc_aa_bwd(const real* color, int C, const real* rast, const real* pos, long pos_view_stride, long V,
                          const int32_t* tri, long F, const int32_t* nbr, int B, int H, int W, const real* grad_out,
                          real boost, real* grad_color, double* grad_pos, int nthreads) {
    (void)F;
    if (C > ORC_MAX_AA_CHANNELS) return 2;
    long npix = (long)H * W;
    int nt = max_threads(nthreads);
    long gsize = (pos_view_stride ? (long)B : 1) * V * 4;
    double* acc = (double*)calloc((size_t)nt * (size_t)gsize, sizeof(double));
    if (!acc) return 1;
#pragma omp parallel num_threads(nt)
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        double* Acc = acc + (size_t)tid * (size_t)gsize;
#pragma omp for schedule(static)
        for (long i = 0; i < (long)B * npix; ++i) {
            int b = (int)(i / npix);
            long pix = i % npix;
            int py = (int)(pix / W), px = (int)(pix % W);
            const real* R = rast + (size_t)b * (size_t)npix * 4;
            const real* Cc = color + (size_t)b * (size_t)npix * C;
            const real* Gd = grad_out + (size_t)b * (size_t)npix * C;
            const real* P = pos + (size_t)b * (size_t)pos_view_stride;
            double* GP = Acc + (pos_view_stride ? (size_t)b * (size_t)V * 4 : 0);
            double gc[ORC_MAX_AA_CHANNELS];
            int CC = C;
            for (int c = 0; c < CC; ++c) gc[c] = Gd[pix * C + c];
            long pairs[4][2];
            int np = 0;
            if (px > 0) { pairs[np][0] = pix - 1; pairs[np][1] = pix; ++np; }
            if (px < W - 1) { pairs[np][0] = pix; pairs[np][1] = pix + 1; ++np; }
            if (py > 0) { pairs[np][0] = pix - W; pairs[np][1] = pix; ++np; }
            if (py < H - 1) { pairs[np][0] = pix; pairs[np][1] = pix + W; ++np; }
            for (int q = 0; q < np; ++q) {
                aa_pair_t pr;
                aa_pair(R, P, tri, nbr, W, H, pairs[q][0], pairs[q][1], &pr);
                if (!pr.valid) continue;
                if (pr.target == pix)
                    for (int c = 0; c < CC; ++c) gc[c] -= (double)pr.w * Gd[pix * C + c];
                if (pr.src == pix)
                    for (int c = 0; c < CC; ++c) gc[c] += (double)pr.w * Gd[pr.target * C + c];
                /* position gradient: each pair once, owned by its first pixel */
                if (pairs[q][0] != pix || pr.clamped) continue;
                double dLdw = 0;
                for (int c = 0; c < C; ++c)
                    dLdw += (double)Gd[pr.target * C + c] * ((double)Cc[pr.src * C + c] - (double)Cc[pr.target * C + c]);
                double dLdt = dLdw * pr.sign * (double)boost;
                double den = (double)pr.eF - (double)pr.eO;
                double dt_deF = -(double)pr.eO / (den * den);
                double dt_deO = (double)pr.eF / (den * den);
                const real* a = pr.s[(pr.k + 1) % 3];
                const real* bb = pr.s[(pr.k + 2) % 3];
                double gA[2] = {0, 0}, gB[2] = {0, 0};
                const real* cs[2] = {pr.cF, pr.cO};
                double dts[2] = {dt_deF, dt_deO};
                for (int m = 0; m < 2; ++m) {
                    const real* p = cs[m];
                    double f = dLdt * dts[m] * (double)pr.sgn;
                    gA[0] += f * ((double)bb[1] - (double)p[1]);
                    gA[1] += f * ((double)p[0] - (double)bb[0]);
                    gB[0] += f * ((double)p[1] - (double)a[1]);
                    gB[1] += f * ((double)a[0] - (double)p[0]);
                }
                const int32_t* ti = tri + (size_t)pr.T * 3;
                int32_t vi[2] = {ti[(pr.k + 1) % 3], ti[(pr.k + 2) % 3]};
                double* gs[2] = {gA, gB};
                for (int m = 0; m < 2; ++m) {
                    const real* pv = P + (size_t)vi[m] * 4;
                    double x = pv[0], y = pv[1], w = pv[3];
                    double hx = 0.5 * W, hy = 0.5 * H;
                    double* g = GP + (size_t)vi[m] * 4;
                    g[0] += gs[m][0] * hx / w;
                    g[1] += gs[m][1] * hy / w;
                    g[3] += -(gs[m][0] * hx * x + gs[m][1] * hy * y) / (w * w);
                }
            }
            for (int c = 0; c < CC; ++c) grad_color[i * C + c] = (real)gc[c];
        }
    }
    for (int th = 0; th < nt; ++th)
        for (long j = 0; j < gsize; ++j) grad_pos[j] += acc[(size_t)th * (size_t)gsize + j];
    free(acc);
    return ORC_OK;
}

/* ---------------------------------------------------------------------- */
/* Finite-difference support: the L1 loss with visibility held fixed.      */
/* ---------------------------------------------------------------------- */
/*
 * The gradients diffrp gets from dr.antialias (diffrp/rendering/
 * surface_deferred.py:775) and from the interpolation autograd
 * (diffrp/rendering/interpolator.py:32-48) are those of the image with every
 * discrete decision of the forward held: each pixel's triangle, and for each
 * antialias pair the front triangle, the crossing edge, which pixel is
 * blended and whether its crossing parameter was clamped.  Central
 * differences of the loss evaluated that way check the analytic backward
 * (rasterisation, interpolation, antialias silhouette term) without the
 * discontinuities of coverage changes.
 *
 * orc_aa_plan lists the decisions of one view's antialias forward, evaluated
 * in this build's precision (use the float build: its decisions are those of
 * the CUDA forward, bit for bit).  One entry per valid pair, 8 int32 each:
 *   target pixel, source pixel, front pixel, other pixel, front triangle,
 *   crossing edge k, branch (+1: w = t - 1/2, -1: w = 1/2 - t, 0: t clamped,
 *   w = 1/2 fixed), orientation sign of the front triangle (+1 / -1).
 * Returns the number of entries; writes at most cap of them.
 */
ORC_EXPORT long orc_aa_plan(const real* rast, const real* pos, long V, const int32_t* tri, long F,
                            const int32_t* nbr, int H, int W, int32_t* plan, long cap) {
    (void)V; (void)F;
    long n = 0;
    long npix = (long)H * W;
    for (long pix = 0; pix < npix; ++pix) {
        int px = (int)(pix % W), py = (int)(pix / W);
        long pairs[2][2];
        int np = 0;
        if (px < W - 1) { pairs[np][0] = pix; pairs[np][1] = pix + 1; ++np; }
        if (py < H - 1) { pairs[np][0] = pix; pairs[np][1] = pix + W; ++np; }
        for (int q = 0; q < np; ++q) {
            aa_pair_t pr;
            aa_pair(rast, pos, tri, nbr, W, H, pairs[q][0], pairs[q][1], &pr);
            if (!pr.valid) continue;
            if (n < cap) {
                int32_t* e = plan + n * 8;
                e[0] = (int32_t)pr.target;
                e[1] = (int32_t)pr.src;
                /* front pixel: the pixel holding T */
                e[2] = rast_tri(rast + pairs[q][0] * 4) == pr.T ? (int32_t)pairs[q][0] : (int32_t)pairs[q][1];
                e[3] = e[2] == (int32_t)pairs[q][0] ? (int32_t)pairs[q][1] : (int32_t)pairs[q][0];
                e[4] = pr.T;
                e[5] = pr.k;
                e[6] = pr.clamped ? 0 : (int32_t)pr.sign;
                e[7] = pr.sgn > 0 ? 1 : -1;
            }
            ++n;
        }
    }
    return n;
}

static inline void pixel_color(const real* pos, const int32_t* tri, const real* attr, int C, int t, long pix, int H,
                               int W, real* col) {
    const int32_t* ti = tri + (size_t)t * 3;
    shade_t S;
    shade_eval(pos + (size_t)ti[0] * 4, pos + (size_t)ti[1] * 4, pos + (size_t)ti[2] * 4, (int)(pix % W),
               (int)(pix / W), W, H, &S);
    const real* a0 = attr + (size_t)ti[0] * C;
    const real* a1 = attr + (size_t)ti[1] * C;
    const real* a2 = attr + (size_t)ti[2] * C;
    for (int c = 0; c < C; ++c) col[c] = r_fma(a0[c] - a2[c], S.u, r_fma(a1[c] - a2[c], S.v, a2[c]));
}

/*
 * sum over pixels and channels of sign * out, with out the antialiased
 * interpolation of attr under the fixed decisions: ids (per pixel triangle
 * or -1) and the plan of orc_aa_plan.  sign is the per (pixel, channel) sign
 * of (out - target) at the point the gradient is taken (the L1 loss
 * linearised at its kinks the way its gradient is).  With tri_flag (one
 * byte per triangle) only the terms that involve a flagged triangle are
 * summed: the pixels of flagged triangles, and the pairs whose front
 * triangle or either pixel's triangle is flagged.  Every other term does
 * not depend on the vertices of the flagged triangles, so differences of
 * two evaluations equal those of the full sum.  Single view.
 */
ORC_EXPORT int orc_l1_fixed_visibility(const real* pos, const int32_t* tri, const real* attr, int C, int H, int W,
                                       const int32_t* ids, const int8_t* sign, const int32_t* plan, long n_plan,
                                       const uint8_t* tri_flag, double* result, int nthreads) {
    if (C > ORC_MAX_AA_CHANNELS) return 2;
    long npix = (long)H * W;
    /* per-thread partial sums over static chunks, added in thread order: the
       same inputs give the same bits (differences of two evaluations that
       change no term are exactly zero) */
    int nt = max_threads(nthreads);
    double* part = (double*)calloc((size_t)nt, sizeof(double));
    if (!part) return 1;
#pragma omp parallel num_threads(nt)
    {
        real col[ORC_MAX_AA_CHANNELS], cs[ORC_MAX_AA_CHANNELS];
        double total = 0.0;
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
#pragma omp for schedule(static)
        for (long pix = 0; pix < npix; ++pix) {
            int t = ids[pix];
            if (t < 0 || (tri_flag && !tri_flag[t])) continue;
            pixel_color(pos, tri, attr, C, t, pix, H, W, col);
            for (int c = 0; c < C; ++c) total += (double)sign[pix * C + c] * (double)col[c];
        }
#pragma omp for schedule(static)
        for (long e = 0; e < n_plan; ++e) {
            const int32_t* p = plan + e * 8;
            long tgt = p[0], src = p[1], Fp = p[2], Op = p[3];
            int T = p[4], k = p[5], branch = p[6];
            real sgn = (real)p[7];
            int tt = ids[tgt], ts = ids[src];
            if (tri_flag && !tri_flag[T] && !(tt >= 0 && tri_flag[tt]) && !(ts >= 0 && tri_flag[ts])) continue;
            real w = (real)0.5;
            if (branch != 0) {
                const int32_t* ti = tri + (size_t)T * 3;
                real s[3][2];
                int ok = 1;
                for (int i = 0; i < 3; ++i) ok &= project_vertex(pos + (size_t)ti[i] * 4, W, H, s[i]);
                if (!ok) continue;
                real cF[2] = {(real)(Fp % W) + (real)0.5, (real)(Fp / W) + (real)0.5};
                real cO[2] = {(real)(Op % W) + (real)0.5, (real)(Op / W) + (real)0.5};
                const real* a = s[(k + 1) % 3];
                const real* b = s[(k + 2) % 3];
                real eF = sgn * edge_fn(a, b, cF), eO = sgn * edge_fn(a, b, cO);
                real tc = eF / (eF - eO);
                w = branch > 0 ? tc - (real)0.5 : (real)0.5 - tc;
            }
            for (int c = 0; c < C; ++c) col[c] = 0, cs[c] = 0;
            if (tt >= 0) pixel_color(pos, tri, attr, C, tt, tgt, H, W, col);
            if (ts >= 0) pixel_color(pos, tri, attr, C, ts, src, H, W, cs);
            for (int c = 0; c < C; ++c) total += (double)sign[tgt * C + c] * (double)(w * (cs[c] - col[c]));
        }
        part[tid] = total;
    }
    double total = 0.0;
    for (int i = 0; i < nt; ++i) total += part[i];
    free(part);
    *result = total;
    return ORC_OK;
}
