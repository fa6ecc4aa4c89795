// FP32 Newtonian sweeps on cell pairs: every thread carries two cells through Blackwell's paired
// FP32 instructions (FFMA2 / FADD2 / FMUL2) and moves them with 8-byte loads and stores.  The
// arithmetic is physics_fast.cuh's, instantiated on the pair type, so the results equal the
// one-cell kernels' bit for bit.
#pragma once
#include "physics_fast.cuh"
#include "sweep_kernels.cuh"

namespace cg {

struct Cell2 {
    f2 v[5];
};

// Y sweep: one thread marches rows y0 .. y0 + SEG - 1 of columns j, j + 1 (j even) with the
// stencil in registers, loading each row one iteration ahead; every interface flux is computed
// once.  A lone last column (odd nx) runs in both lanes.
template <int LIM, int NT, int SEG>
__global__ void __launch_bounds__(NT) sweep_y_pair_kernel(NewtonFastParams P, int dims, Geom G,
                                                          const float* __restrict__ src, float* __restrict__ dst,
                                                          DtSrc ds, SweepOut out) {
    __shared__ FastCoef s_coef;
    __shared__ int s_act;
    if (threadIdx.x == 0) {
        double dt;
        s_act = ds.get(dt);
        if (s_act) s_coef = ds.fast_coef();
    }
    __syncthreads();
    const bool act = s_act != 0;
    const int j = 2 * (blockIdx.x * NT + threadIdx.x);
    const int n = G.ny;
    const int y0 = blockIdx.y * SEG, y1 = min(y0 + SEG, n);
    const bool col_ok = j < G.nx, two = j + 1 < G.nx;
    unsigned long long* wslot = out.slot();
    float w = 0.0f;
    auto ld = [&](int y, Cell2& c) {
        const size_t b = (size_t)ghost_index(y, n, G.bc) * G.pitch + j;
#pragma unroll
        for (int f = 0; f < 5; f++) {
            const float* p = src + f * G.fstride + b;
            if (two) {
                c.v[f].v = *reinterpret_cast<const float2*>(p);
            } else {
                const float x = *p;
                c.v[f].v = make_float2(x, x);
            }
        }
    };
    auto st = [&](int y, const Cell2& c) {
        const size_t b = (size_t)y * G.pitch + j;
#pragma unroll
        for (int f = 0; f < 5; f++) {
            float* p = dst + f * G.fstride + b;
            if (two) *reinterpret_cast<float2*>(p) = c.v[f].v;
            else *p = c.v[f].v.x;
        }
    };
    if (col_ok) {
        if (!act) {
            for (int y = y0; y < y1; y++) {
                Cell2 c;
                ld(y, c);
                st(y, c);
            }
        } else {
            const FastCoef cf = s_coef;
            Cell2 cm2, cm1, c0, c1, c2, ahead;
            ld(y0 - 2, cm2);
            ld(y0 - 1, cm1);
            ld(y0, c0);
            ld(y0 + 1, c1);
            ld(y0 + 2, ahead);
            f2 Lm1[5], Rm1[5], L0[5], R0[5], Fp[5], Fn[5];
            nf_recon<1, LIM>(P, cm2.v, cm1.v, c0.v, cf.half_dtdx, Lm1, Rm1);
            nf_recon<1, LIM>(P, cm1.v, c0.v, c1.v, cf.half_dtdx, L0, R0);
            nf_force<1>(P, Rm1, L0, cf.half_dtdx, cf.q_dxdt, Fp);
            for (int y = y0; y < y1; y++) {
                // the next row is loaded one iteration ahead, so its latency overlaps this row's work
                c2 = ahead;
                if (y + 1 < y1) ld(y + 3, ahead);
                f2 L1[5], R1[5];
                nf_recon<1, LIM>(P, c0.v, c1.v, c2.v, cf.half_dtdx, L1, R1);
                nf_force<1>(P, R0, L1, cf.half_dtdx, cf.q_dxdt, Fn);
                Cell2 nc;
                nf_update(cf.dtdx, c0.v, Fp, Fn, nc.v);
                st(y, nc);
                if (wslot) {
                    const f2 ws = nf_wavespeed(P, nc.v, dims);
                    // fmaxf drops a NaN (as the one-cell kernels' `ws > w` does); a lone column's
                    // duplicated lane repeats the same value
                    w = fmaxf(w, fmaxf(ws.v.x, ws.v.y));
                }
#pragma unroll
                for (int f = 0; f < 5; f++) {
                    Fp[f] = Fn[f];
                    R0[f] = R1[f];
                }
                c0 = c1;
                c1 = c2;
            }
        }
    }
    if (wslot) block_max_to<NT>(wslot, w);
}

// X sweep on row segments of 64 cells: lane t holds the cells at positions s0 - 2 + 2t and
// s0 - 1 + 2t.  Neighbour cells, the next cell's left face state and the previous cell pair's
// right-face flux cross lanes by warp shuffles, so no shared memory and no block barrier is used;
// lanes 1..30 update their two cells (60 cells per segment; the two cells at each end are the
// stencil halo).  A warp walks SEGS consecutive segments of its row, loading the next segment
// while it computes the current one.
template <int LIM, int NT, int SEGS>
__global__ void __launch_bounds__(NT) sweep_x_pair_kernel(NewtonFastParams P, int dims, Geom G,
                                                          const float* __restrict__ src, float* __restrict__ dst,
                                                          DtSrc ds, SweepOut out) {
    constexpr unsigned FULL = 0xffffffffu;
    constexpr int TSW = 60;
    __shared__ FastCoef s_coef;
    __shared__ int s_act;
    if (threadIdx.x == 0) {
        double dt;
        s_act = ds.get(dt);
        if (s_act) s_coef = ds.fast_coef();
    }
    __syncthreads();
    const bool act = s_act != 0;
    const int lane = threadIdx.x & 31;
    const int seg0 = (blockIdx.x * (NT / 32) + (threadIdx.x >> 5)) * SEGS;
    const int row = blockIdx.y;
    const int n = G.nx;
    const size_t rb = (size_t)row * G.pitch;
    unsigned long long* wslot = out.slot();
    float w = 0.0f;
    auto ld = [&](int s0, Cell2& m) {
        const int p0 = s0 - 2 + 2 * lane;
        if (p0 >= 0 && p0 + 1 < n) {
#pragma unroll
            for (int f = 0; f < 5; f++) m.v[f].v = *reinterpret_cast<const float2*>(src + f * G.fstride + rb + p0);
        } else {
            // ghost positions (at most two outside the row are used; further ones only feed the
            // discarded halo work and are clamped to a valid ghost)
            const int qa = ghost_index(min(p0, n + 1), n, G.bc), qb = ghost_index(min(p0 + 1, n + 1), n, G.bc);
#pragma unroll
            for (int f = 0; f < 5; f++) m.v[f].v = make_float2(src[f * G.fstride + rb + qa], src[f * G.fstride + rb + qb]);
        }
    };
    Cell2 ahead;
    if (seg0 * TSW < n) ld(seg0 * TSW, ahead);
    for (int k = 0; k < SEGS; k++) {
        const int s0 = (seg0 + k) * TSW;
        if (s0 >= n) break;  // warp-uniform
        Cell2 m = ahead;
        if (k + 1 < SEGS && s0 + TSW < n) ld(s0 + TSW, ahead);
        const int p0 = s0 - 2 + 2 * lane;
        const bool upd = lane >= 1 && lane <= 30;
        Cell2 nc = m;
        if (act) {
            const FastCoef cf = s_coef;
            f2 l[5], r[5];
#pragma unroll
            for (int f = 0; f < 5; f++) {
                l[f].v = make_float2(__shfl_up_sync(FULL, m.v[f].v.y, 1), m.v[f].v.x);
                r[f].v = make_float2(m.v[f].v.y, __shfl_down_sync(FULL, m.v[f].v.x, 1));
            }
            f2 L[5], R[5];
            nf_recon<0, LIM>(P, l, m.v, r, cf.half_dtdx, L, R);
            f2 Rn[5];  // left face states of the cells right of this lane's two
#pragma unroll
            for (int f = 0; f < 5; f++) Rn[f].v = make_float2(L[f].v.y, __shfl_down_sync(FULL, L[f].v.x, 1));
            f2 Fr[5], Fl[5];
            nf_force<0>(P, R, Rn, cf.half_dtdx, cf.q_dxdt, Fr);
#pragma unroll
            for (int f = 0; f < 5; f++) Fl[f].v = make_float2(__shfl_up_sync(FULL, Fr[f].v.y, 1), Fr[f].v.x);
            nf_update(cf.dtdx, m.v, Fl, Fr, nc.v);
        }
        if (upd && p0 < n) {
            if (p0 + 1 < n) {
#pragma unroll
                for (int f = 0; f < 5; f++) *reinterpret_cast<float2*>(dst + f * G.fstride + rb + p0) = nc.v[f].v;
            } else {
#pragma unroll
                for (int f = 0; f < 5; f++) dst[f * G.fstride + rb + p0] = nc.v[f].v.x;
            }
            if (wslot && act) {
                const f2 ws = nf_wavespeed(P, nc.v, dims);
                w = fmaxf(w, p0 + 1 < n ? fmaxf(ws.v.x, ws.v.y) : ws.v.x);
            }
        }
    }
    if (wslot) block_max_to<NT>(wslot, w);
}

}  // namespace cg
