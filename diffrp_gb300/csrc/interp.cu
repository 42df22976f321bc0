// interp.cu -- attribute interpolation forward/backward.
//
// Full-screen form replaces dr.interpolate (diffrp/rendering/interpolator.py:83);
// the sparse form replaces the torch gather + FMA of the stencil-masked
// interpolator (diffrp/rendering/interpolator.py:32-48, 87-97).  Both evaluate
//     out = fma(a0 - a2, u, fma(a1 - a2, v, a2))
// in that order (interpolator.py:45), one thread per pixel, with 128-bit
// vectorised attribute gathers and stores when the channel count is a multiple
// of four.  The backward scatters attribute gradients with float4 atomics
// after a warp-segmented reduction over runs of pixels that share a triangle.
#include "drp_common.cuh"
#include "drp_internal.h"

namespace drp {

__device__ __forceinline__ float4 lerp_attr4(const float4& a0, const float4& a1, const float4& a2, float u, float v) {
    float4 o;
    o.x = fmaf(a0.x - a2.x, u, fmaf(a1.x - a2.x, v, a2.x));
    o.y = fmaf(a0.y - a2.y, u, fmaf(a1.y - a2.y, v, a2.y));
    o.z = fmaf(a0.z - a2.z, u, fmaf(a1.z - a2.z, v, a2.z));
    o.w = fmaf(a0.w - a2.w, u, fmaf(a1.w - a2.w, v, a2.w));
    return o;
}

__global__ void __launch_bounds__(256) interp_fwd_kernel(InterpArgs a) {
    const long long npix_view = (long long)a.H * a.W;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)a.B * npix_view) return;
    const int b = (int)(i / npix_view);
    const float4 r = reinterpret_cast<const float4*>(a.rast)[i];
    int j0 = 0, j1 = 0, j2 = 0;
    const int t = checked_tri(r.w, a.tri, a.num_triangles, a.num_vertices, j0, j1, j2);
    const int C = a.C;
    float* o = a.out + i * C;
    float* dd = a.da ? a.da + i * 2 * a.nd : nullptr;
    if (t < 0) {
        if ((C & 3) == 0) {
            for (int c = 0; c < C; c += 4) *reinterpret_cast<float4*>(o + c) = make_float4(0.f, 0.f, 0.f, 0.f);
        } else {
            for (int c = 0; c < C; ++c) o[c] = 0.f;
        }
        if (dd)
            for (int c = 0; c < 2 * a.nd; ++c) dd[c] = 0.f;
        return;
    }
    const float* A = a.attr + (long long)b * a.attr_view_stride;
    const long long i0 = j0, i1 = j1, i2 = j2;
    const float* a0 = A + i0 * C;
    const float* a1 = A + i1 * C;
    const float* a2 = A + i2 * C;
    const float u = r.x, v = r.y;
    if ((C & 3) == 0) {
        for (int c = 0; c < C; c += 4) {
            const float4 x0 = __ldg(reinterpret_cast<const float4*>(a0 + c));
            const float4 x1 = __ldg(reinterpret_cast<const float4*>(a1 + c));
            const float4 x2 = __ldg(reinterpret_cast<const float4*>(a2 + c));
            *reinterpret_cast<float4*>(o + c) = lerp_attr4(x0, x1, x2, u, v);
        }
    } else {
        for (int c = 0; c < C; ++c) {
            const float x0 = __ldg(a0 + c), x1 = __ldg(a1 + c), x2 = __ldg(a2 + c);
            o[c] = fmaf(x0 - x2, u, fmaf(x1 - x2, v, x2));
        }
    }
    if (dd) {
        const float4 db = reinterpret_cast<const float4*>(a.rast_db)[i];
        for (int k = 0; k < a.nd; ++k) {
            const int c = a.diff_idx[k];
            const float e0 = a0[c] - a2[c], e1 = a1[c] - a2[c];
            dd[2 * k + 0] = fmaf(e0, db.x, e1 * db.z);
            dd[2 * k + 1] = fmaf(e0, db.y, e1 * db.w);
        }
    }
}

__global__ void __launch_bounds__(256) interp_bwd_kernel(InterpArgs a) {
    const long long npix_view = (long long)a.H * a.W;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool in = i < (long long)a.B * npix_view;
    const int b = in ? (int)(i / npix_view) : 0;
    float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
    if (in) r = reinterpret_cast<const float4*>(a.rast)[i];
    int j0 = 0, j1 = 0, j2 = 0;
    const int t = in ? checked_tri(r.w, a.tri, a.num_triangles, a.num_vertices, j0, j1, j2) : -1;
    const int C = a.C;
    const float* A = a.attr + (long long)b * a.attr_view_stride;
    float* G = a.grad_attr + (long long)b * a.attr_view_stride;
    const long long i0 = j0, i1 = j1, i2 = j2;
    const float u = r.x, v = r.y, w = 1.0f - u - v;
    const float* g = a.grad_out + (in ? i : 0) * C;
    float4 db = make_float4(0.f, 0.f, 0.f, 0.f);
    const float* gdd = nullptr;
    if (t >= 0 && a.nd > 0 && a.grad_da) {
        db = reinterpret_cast<const float4*>(a.rast_db)[i];
        gdd = a.grad_da + i * 2 * a.nd;
    }
    const long long key = (t >= 0) ? (a.attr_view_stride ? (((long long)b << 32) | (long long)t) : (long long)t)
                                   : (long long)(-1 - lane_id());
    const Seg seg = seg_setup(key);
    float gu = 0.f, gv = 0.f;
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
    for (int c0 = 0; c0 < C; c0 += 4) {
        float val[12];
#pragma unroll
        for (int k = 0; k < 12; ++k) val[k] = 0.f;
        if (t >= 0) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int c = c0 + k;
                if (c < C) {
                    const float gc = g[c];
                    float w0 = gc * u, w1 = gc * v, w2 = gc * w;
                    const float x0 = A[i0 * C + c], x1 = A[i1 * C + c], x2 = A[i2 * C + c];
                    gu = fmaf(gc, x0 - x2, gu);
                    gv = fmaf(gc, x1 - x2, gv);
                    if (gdd) {
                        for (int q = 0; q < a.nd; ++q) {
                            if (a.diff_idx[q] != c) continue;
                            const float gx = gdd[2 * q], gy = gdd[2 * q + 1];
                            const float d0 = fmaf(gx, db.x, gy * db.y), d1 = fmaf(gx, db.z, gy * db.w);
                            w0 += d0;
                            w1 += d1;
                            w2 -= d0 + d1;
                            s0 = fmaf(gx, x0 - x2, s0);
                            s1 = fmaf(gy, x0 - x2, s1);
                            s2 = fmaf(gx, x1 - x2, s2);
                            s3 = fmaf(gy, x1 - x2, s3);
                        }
                    }
                    val[k] = w0;
                    val[4 + k] = w1;
                    val[8 + k] = w2;
                }
            }
        }
        seg_reduce<12>(seg, val);
        if (t >= 0 && seg.head) {
            if ((C & 3) == 0) {
                atomic_add4(reinterpret_cast<float4*>(G + i0 * C + c0), make_float4(val[0], val[1], val[2], val[3]));
                atomic_add4(reinterpret_cast<float4*>(G + i1 * C + c0), make_float4(val[4], val[5], val[6], val[7]));
                atomic_add4(reinterpret_cast<float4*>(G + i2 * C + c0), make_float4(val[8], val[9], val[10], val[11]));
            } else {
                for (int k = 0; k < 4 && c0 + k < C; ++k) {
                    atomicAdd(G + i0 * C + c0 + k, val[k]);
                    atomicAdd(G + i1 * C + c0 + k, val[4 + k]);
                    atomicAdd(G + i2 * C + c0 + k, val[8 + k]);
                }
            }
        }
    }
    if (in) {
        if (a.grad_rast) reinterpret_cast<float4*>(a.grad_rast)[i] = make_float4(gu, gv, 0.f, 0.f);
        if (a.grad_db) reinterpret_cast<float4*>(a.grad_db)[i] = make_float4(s0, s1, s2, s3);
    }
}

// Sparse form: vi (N, 4) rast rows, tri_idx (N, 3) int64 vertex indices.
__global__ void __launch_bounds__(256) interp_sparse_fwd_kernel(SparseInterpArgs a) {
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= a.N) return;
    const int C = a.C;
    const float4 r = reinterpret_cast<const float4*>(a.vi)[n];
    const long long i0 = a.tri_idx[3 * n], i1 = a.tri_idx[3 * n + 1], i2 = a.tri_idx[3 * n + 2];
    float* o = a.out + n * C;
    if (i0 < 0 || i1 < 0 || i2 < 0 || i0 >= a.V || i1 >= a.V || i2 >= a.V) {
        for (int c = 0; c < C; ++c) o[c] = __int_as_float(0x7fc00000);
        return;
    }
    const float* a0 = a.vb + i0 * C;
    const float* a1 = a.vb + i1 * C;
    const float* a2 = a.vb + i2 * C;
    if ((C & 3) == 0) {
        for (int c = 0; c < C; c += 4) {
            const float4 x0 = __ldg(reinterpret_cast<const float4*>(a0 + c));
            const float4 x1 = __ldg(reinterpret_cast<const float4*>(a1 + c));
            const float4 x2 = __ldg(reinterpret_cast<const float4*>(a2 + c));
            *reinterpret_cast<float4*>(o + c) = lerp_attr4(x0, x1, x2, r.x, r.y);
        }
    } else {
        for (int c = 0; c < C; ++c) {
            const float x0 = __ldg(a0 + c), x1 = __ldg(a1 + c), x2 = __ldg(a2 + c);
            o[c] = fmaf(x0 - x2, r.x, fmaf(x1 - x2, r.y, x2));
        }
    }
}

__global__ void __launch_bounds__(256) interp_sparse_bwd_kernel(SparseInterpArgs a) {
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    bool in = n < a.N;
    const int C = a.C;
    float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
    long long i0 = 0, i1 = 0, i2 = 0;
    if (in) {
        r = reinterpret_cast<const float4*>(a.vi)[n];
        i0 = a.tri_idx[3 * n];
        i1 = a.tri_idx[3 * n + 1];
        i2 = a.tri_idx[3 * n + 2];
        if (i0 < 0 || i1 < 0 || i2 < 0 || i0 >= a.V || i1 >= a.V || i2 >= a.V) {
            in = false;
            i0 = i1 = i2 = 0;
            if (a.grad_vi) reinterpret_cast<float4*>(a.grad_vi)[n] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
    // Runs keyed by the first vertex index of the row's triangle.
    const long long key = in ? (i0 ^ (i1 << 21) ^ (i2 << 42)) : (long long)(-1 - lane_id());
    const Seg seg = seg_setup(key);
    const float u = r.x, v = r.y, w = 1.0f - u - v;
    float gu = 0.f, gv = 0.f;
    for (int c0 = 0; c0 < C; c0 += 4) {
        float val[12];
#pragma unroll
        for (int k = 0; k < 12; ++k) val[k] = 0.f;
        if (in) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int c = c0 + k;
                if (c < C) {
                    const float gc = a.grad_out[n * C + c];
                    const float x0 = a.vb[i0 * C + c], x1 = a.vb[i1 * C + c], x2 = a.vb[i2 * C + c];
                    val[k] = gc * u;
                    val[4 + k] = gc * v;
                    val[8 + k] = gc * w;
                    gu = fmaf(gc, x0 - x2, gu);
                    gv = fmaf(gc, x1 - x2, gv);
                }
            }
        }
        seg_reduce<12>(seg, val);
        if (in && seg.head) {
            for (int k = 0; k < 4 && c0 + k < C; ++k) {
                atomicAdd(a.grad_vb + i0 * C + c0 + k, val[k]);
                atomicAdd(a.grad_vb + i1 * C + c0 + k, val[4 + k]);
                atomicAdd(a.grad_vb + i2 * C + c0 + k, val[8 + k]);
            }
        }
    }
    if (in && a.grad_vi) reinterpret_cast<float4*>(a.grad_vi)[n] = make_float4(gu, gv, 0.f, 0.f);
}

int launch_interp_fwd(const InterpArgs& a, cudaStream_t s) {
    const long long n = (long long)a.B * a.H * a.W;
    if (n == 0) return 0;
    interp_fwd_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a);
    drp_note_launch();
    return 0;
}

int launch_interp_bwd(const InterpArgs& a, cudaStream_t s) {
    const long long n = (long long)a.B * a.H * a.W;
    if (n == 0) return 0;
    interp_bwd_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a);
    drp_note_launch();
    return 0;
}

int launch_interp_sparse_fwd(const SparseInterpArgs& a, cudaStream_t s) {
    if (a.N == 0) return 0;
    interp_sparse_fwd_kernel<<<(unsigned)((a.N + 255) / 256), 256, 0, s>>>(a);
    drp_note_launch();
    return 0;
}

int launch_interp_sparse_bwd(const SparseInterpArgs& a, cudaStream_t s) {
    if (a.N == 0) return 0;
    interp_sparse_bwd_kernel<<<(unsigned)((a.N + 255) / 256), 256, 0, s>>>(a);
    drp_note_launch();
    return 0;
}

}  // namespace drp
