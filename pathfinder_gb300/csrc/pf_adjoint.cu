// pf_adjoint.cu — the adjoint of a differentiable frame.
//
// The reference has no backward pass; this is the added differentiable mode
// of the CUDA level.  The forward (k_composite_diff) renders single-channel
// FP32 coverage from FP32 fills and records, per visible entry and pixel, the
// coverage c, the composite value d below the entry and dc/dmask.  Here:
//
// 1. k_composite_bwd (one warp per screen tile) walks each tile's list in
//    reverse draw order.  SrcOver d' = a + d (1 - a) with a = alpha * c gives
//    dL/da = G (1 - d) and G <- G (1 - a); dL/dalpha += dL/da * c and
//    dL/dmask += dL/da * alpha * dc/dmask, per alpha tile and pixel.
//
// 2. k_line_grad (one thread per flattened line, binning recomputed instead
//    of stored per-tile fill lists) maps dL/dmask onto the line's endpoints.
//    A pixel's mask value w is the integral of the path's winding number
//    over the pixel: the sum over fills of the trapezoid area below each fill
//    plus the backdrop (fill_area.inc.glsl:11-27, tiler.rs:191-308).  For a
//    closed path that is exact, so tile clipping, auxiliary fills and
//    backdrops drop out of its first variation: moving the line
//    P(u) = A + u (B - A) by dP changes w(pixel) by the integral over the part
//    of the line inside the pixel of dP . n du, n = (-(B-A).y, (B-A).x).  With
//    dP = (1-u) dA + u dB, over u in [u0, u1]:
//        dw/dA = n * I0,  I0 = (u1-u0) - (u1^2-u0^2)/2
//        dw/dB = n * I1,  I1 = (u1^2-u0^2)/2.
//    The line is walked pixel by pixel (a unit-grid DDA) over the pixels of
//    its path's tiles that lie inside the view box.
//
// 3. The line's ends are curve points at the recorded parameters t0, t1 (the
//    subdivision stays fixed), so dL/dP_i = b_i(t0) dL/dA + b_i(t1) dL/dB
//    with the Bernstein weights of the segment (quadratics through the
//    degree elevation of Segment::to_cubic, content/src/segment.rs:171-182).
//    Lines of one segment are consecutive, so a warp sums its lanes per
//    segment and one lane per segment issues the atomics.
#include "pf_kernels.cuh"

namespace pf {

// ---------------------------------------------------------------------------
// 1. composite adjoint
// ---------------------------------------------------------------------------
template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32) k_composite_bwd(FrameDev f, const float* __restrict__ dimg,
                                                               float* grad_mask, float* grad_alpha) {
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t st = blockIdx.x * WARPS + wid;
    if (st >= f.screen_count) return;
    if (!(frame_ok(f) && f.counters->fills <= f.fill_cap && f.counters->visible <= f.vis_cap)) return;
    const uint32_t base = f.screen_base[st], n = f.screen_base[st + 1] - base;
    if (n == 0) return;

    const SceneDev& sc = f.scenes[scene_of_screen_tile(f, f.screen_begin + st)];
    const int4 s = sc.screen;
    const int32_t sw = s.z - s.x;
    const uint32_t lst = f.screen_begin + st - sc.screen_offset;
    const int32_t tx = s.x + (int32_t)(lst % (uint32_t)sw), ty = s.y + (int32_t)(lst / (uint32_t)sw);
    const int col = lane & 15, half = lane >> 4;
    const int X = tx * 16 + col;

    float G[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const int Y = ty * 16 + half * 8 + k;
        const bool in = X >= sc.clip.x && X < sc.clip.z && Y >= sc.clip.y && Y < sc.clip.w;
        G[k] = in ? dimg[sc.out_offset + (uint64_t)(int64_t)(Y - sc.origin_y) * (uint64_t)(int64_t)sc.pitch +
                         (uint64_t)(int64_t)(X - sc.origin_x)]
                  : 0.0f;
    }
    for (uint32_t i = n; i-- > 0;) {
        const uint32_t e = base + i, g = f.vis[e];
        const int4 rec = f.tiles[g];
        const uint32_t gp = (uint32_t)rec.z, di = f.path.draw_index[gp];
        const float pa = f.path.alpha_f[di];
        uint32_t am = (uint32_t)rec.y, ac = kInvalid;
        if (f.path.clip_gpath[gp] >= 0) {
            const int4 crec = f.clips[g];
            if ((uint32_t)crec.x != kInvalid && (uint32_t)crec.z != kInvalid) { am = (uint32_t)crec.x; ac = (uint32_t)crec.z; }
        }
        const uint64_t t0 = (uint64_t)e * 256u + (uint32_t)(half * 128 + col);
        float ga = 0.0f;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const uint32_t tw = f.tape[t0 + k * 16];
            const float c = tape_cov(tw), dprev = tape_dprev(tw);
            const uint32_t code = tape_code(tw);
            const float dlda = G[k] * (1.0f - dprev);
            ga += dlda * c;
            const float dm = dlda * pa;
            const uint32_t pix = (uint32_t)((half * 8 + k) * 16 + col);
            if (code & 3u) atomicAdd(&grad_mask[(uint64_t)am * 256u + pix], dm * dec_d(code & 3u));
            if (code >> 2) atomicAdd(&grad_mask[(uint64_t)ac * 256u + pix], dm * dec_d(code >> 2));
            G[k] *= 1.0f - pa * c;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) ga += __shfl_xor_sync(0xffffffffu, ga, o);
        if (lane == 0 && ga != 0.0f) atomicAdd(&grad_alpha[di], ga);
    }
}

// Zero dL/dmask for the frame's alpha tiles (count read on the device).
__global__ void k_zero_grad_mask(FrameDev f, float4* grad_mask) {
    if (!frame_ok(f)) return;
    const uint64_t A = f.counters->alpha_tiles;
    if (A > f.tile_cap) return;
    const uint64_t n = A * 64u;  // float4s
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        grad_mask[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

void launch_composite_bwd(const FrameDev& f, const float* d_image, float* grad_mask, float* grad_alpha,
                          cudaStream_t s) {
    count_launch();
    k_zero_grad_mask<<<f.sms * 4, 256, 0, s>>>(f, (float4*)grad_mask);
    if (f.screen_count == 0) return;
    count_launch();
    k_composite_bwd<4><<<(f.screen_count + 3) / 4, 128, 0, s>>>(f, d_image, grad_mask, grad_alpha);
}

// ---------------------------------------------------------------------------
// 2. line adjoint
// ---------------------------------------------------------------------------
// Liang-Barsky step: keep u with p * u <= q.
__device__ __forceinline__ bool lb_clip(float p, float q, float& ua, float& ub) {
    if (p == 0.0f) return q >= 0.0f;
    const float r = q / p;
    if (p < 0.0f) { if (r > ua) ua = r; }
    else if (r < ub) ub = r;
    return true;
}

// Sums over the pixels the line crosses of dL/dmask * I0 and * I1.
__device__ __forceinline__ void line_boundary_sums(const FrameDev& f, float4 ln, uint32_t gp,
                                                   const float* __restrict__ gm, float& GA, float& GB) {
    GA = 0.0f; GB = 0.0f;
    const int4 r = f.path.tile_rect[gp];
    if (r.z <= r.x || r.w <= r.y) return;
    const float4 v = f.scenes[f.path.scene[gp]].view_box;
    // pixels of the path's tiles that lie wholly inside the view box
    const int PX0 = max(r.x * 16, (int)ceilf(v.x)), PX1 = min(r.z * 16, (int)floorf(v.z));
    const int PY0 = max(r.y * 16, (int)ceilf(v.y)), PY1 = min(r.w * 16, (int)floorf(v.w));
    if (PX1 <= PX0 || PY1 <= PY0) return;
    const float x0 = ln.x, y0 = ln.y, dx = ln.z - ln.x, dy = ln.w - ln.y;
    if (dx == 0.0f && dy == 0.0f) return;
    float ua = 0.0f, ub = 1.0f;
    if (!lb_clip(-dx, x0 - (float)PX0, ua, ub) || !lb_clip(dx, (float)PX1 - x0, ua, ub) ||
        !lb_clip(-dy, y0 - (float)PY0, ua, ub) || !lb_clip(dy, (float)PY1 - y0, ua, ub) || !(ua < ub))
        return;
    const uint32_t tbase = f.path.tile_offset[gp];
    const int32_t tw = r.z - r.x;
    const float sx = x0 + ua * dx, sy = y0 + ua * dy;
    int X = (int)floorf(sx), Y = (int)floorf(sy);
    if (dx < 0.0f && (float)X == sx) X--;  // leaving a grid line leftwards: the pixel on its left
    if (dy < 0.0f && (float)Y == sy) Y--;
    const int sX = dx > 0.0f ? 1 : -1, sY = dy > 0.0f ? 1 : -1;
    const float ix = dx != 0.0f ? 1.0f / dx : 0.0f, iy = dy != 0.0f ? 1.0f / dy : 0.0f;
    const uint32_t limit = (uint32_t)min(fabsf(dx) + fabsf(dy) + 4.0f, (float)f.dda_limit);
    float u = ua;
    for (uint32_t it = 0; it < limit; it++) {
        const float ux = dx != 0.0f ? ((float)(X + (dx > 0.0f ? 1 : 0)) - x0) * ix : INFINITY;
        const float uy = dy != 0.0f ? ((float)(Y + (dy > 0.0f ? 1 : 0)) - y0) * iy : INFINITY;
        const float ue = fminf(fminf(ux, uy), ub);
        if (ue > u) {
            if (X >= PX0 && X < PX1 && Y >= PY0 && Y < PY1) {
                const uint32_t g = tbase + (uint32_t)((X >> 4) - r.x) + (uint32_t)tw * (uint32_t)((Y >> 4) - r.y);
                const uint32_t a = (uint32_t)f.tiles[g].y;
                if (a != kInvalid && f.alpha_owner[a] == g) {
                    const float gv = gm[(uint64_t)a * 256u + (uint32_t)((Y & 15) * 16 + (X & 15))];
                    const float du = ue - u, sum = ue + u;
                    GA += gv * du * (1.0f - 0.5f * sum);
                    GB += gv * du * (0.5f * sum);
                }
            }
            u = ue;
        }
        if (ue >= ub) return;
        if (ux <= uy) X += sX; else Y += sY;
    }
    atomicOr(&f.counters->status, kStatusDdaLimit);
}

// Weights of the segment's point slots (first, first+1, first+2, end) at t.
__device__ __forceinline__ void segment_weights(int kind, float t, float w[4]) {
    const float s = 1.0f - t;
    if (kind == (int)kSegCubic) {
        w[0] = s * s * s; w[1] = 3.0f * t * s * s; w[2] = 3.0f * t * t * s; w[3] = t * t * t;
    } else if (kind == (int)kSegQuad) {
        w[0] = s * s; w[1] = 2.0f * t * s; w[2] = 0.0f; w[3] = t * t;
    } else {
        w[0] = s; w[1] = 0.0f; w[2] = 0.0f; w[3] = t;
    }
}

__global__ void __launch_bounds__(256) k_line_grad(FrameDev f, const float* __restrict__ gm, float2* gpts) {
    if (!frame_ok(f)) return;
    const uint64_t Lc = f.counters->lines;
    if (Lc > f.line_cap) return;
    const uint32_t L = (uint32_t)Lc;
    const int lane = threadIdx.x & 31;
    const uint32_t w0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t b = w0 * 32u; b < L; b += nw * 32u) {  // whole warps iterate together
        const uint32_t l = b + (uint32_t)lane;
        uint32_t seg = kInvalid;
        float gx[4] = {0, 0, 0, 0}, gy[4] = {0, 0, 0, 0};
        SegRec sr = make_int4(0, 0, 0, 0);
        if (l < L) {
            seg = f.line_seg[l];
            sr = f.segs[seg];
            const float4 ln = f.lines[l];
            float GA, GB;
            line_boundary_sums(f, ln, f.line_path[l], gm, GA, GB);
            const float nx = -(ln.w - ln.y), ny = ln.z - ln.x;  // n = (-(B-A).y, (B-A).x)
            const float2 t = f.line_t[l];
            float wa[4], wb[4];
            segment_weights(sr.z, t.x, wa);
            segment_weights(sr.z, t.y, wb);
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const float c = wa[i] * GA + wb[i] * GB;
                gx[i] = c * nx;
                gy[i] = c * ny;
            }
        }
        // sum the lanes of each segment (runs of consecutive lanes)
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t so = __shfl_down_sync(0xffffffffu, seg, o);
            float vx[4], vy[4];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                vx[i] = __shfl_down_sync(0xffffffffu, gx[i], o);
                vy[i] = __shfl_down_sync(0xffffffffu, gy[i], o);
            }
            if (lane + o < 32 && so == seg) {
#pragma unroll
                for (int i = 0; i < 4; i++) { gx[i] += vx[i]; gy[i] += vy[i]; }
            }
        }
        const uint32_t sp = __shfl_up_sync(0xffffffffu, seg, 1);
        const bool head = seg != kInvalid && (lane == 0 || sp != seg);
        if (head) {
            const uint32_t idx[4] = {(uint32_t)sr.x, (uint32_t)sr.x + 1u, (uint32_t)sr.x + 2u, (uint32_t)sr.y};
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const bool used =
                    i == 0 || i == 3 || (i == 1 && sr.z != (int)kSegLine) || (i == 2 && sr.z == (int)kSegCubic);
                if (used) {
                    atomicAdd(&gpts[idx[i]].x, gx[i]);
                    atomicAdd(&gpts[idx[i]].y, gy[i]);
                }
            }
        }
    }
}

void launch_line_grad(const FrameDev& f, const float* grad_mask, float2* grad_points, cudaStream_t s) {
    count_launch();
    k_line_grad<<<f.sms * 8, 256, 0, s>>>(f, grad_mask, grad_points);
}

// dL/dp = M^T dL/dp' for p' = M p + t (M = [m00 m01; m10 m11]).
__global__ void k_points_grad_transform(float2* g, uint32_t n, float m00, float m01, float m10, float m11) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float2 v = g[i];
        g[i] = make_float2(m00 * v.x + m10 * v.y, m01 * v.x + m11 * v.y);
    }
}

void launch_points_grad_transform(float2* grad_points, uint32_t n, const float* m4, cudaStream_t s) {
    if (n == 0) return;
    count_launch();
    k_points_grad_transform<<<min((n + 255) / 256, device_sm_count() * 8u), 256, 0, s>>>(grad_points, n, m4[0], m4[1], m4[2], m4[3]);
}

}  // namespace pf
