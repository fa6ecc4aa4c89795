// FP32 Newtonian sweeps on cell pairs: every thread carries two cells through Blackwell's paired
// FP32 instructions (FFMA2 / FADD2 / FMUL2) and moves them with 8-byte loads and stores.  The
// arithmetic is physics_fast.cuh's, instantiated on the pair type; the FORCE flux is taken as four
// times itself (nf_force4), so the results agree with the one-cell kernels' to FP32 rounding.
#pragma once
#include "physics_fast.cuh"
#include "sweep_kernels.cuh"
#include "tma.cuh"

namespace cg {

struct Cell2 {
    f2 v[5];
};

// ---- device functions shared by the single-grid kernels below and the batched launch

// Y march of one thread over rows [y0, y1) of columns j, j + 1 (j even, j < nx) with the stencil
// in registers, loading each row one iteration ahead; every interface flux is computed once.  A
// lone last column (odd nx) runs in both lanes.  Returns the thread's wavespeed maximum over its
// updated cells when want_w (0 otherwise).
template <int LIM>
CG_D float y_pair_march(const NewtonFastParams& P, int dims, const Geom& G, const float* __restrict__ src,
                        float* __restrict__ dst, int j, int y0, int y1, bool act, const FastCoef& cf, bool want_w) {
    const int n = G.ny;
    const bool two = j + 1 < G.nx;
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
    if (!act) {  // inactive step: keep the ping-pong buffers consistent
        for (int y = y0; y < y1; y++) {
            Cell2 c;
            ld(y, c);
            st(y, c);
        }
        return w;
    }
    const Force4Coef c4 = force4_coef(cf);
    Cell2 cm2, cm1, c0, c1, c2, ahead;
    ld(y0 - 2, cm2);
    ld(y0 - 1, cm1);
    ld(y0, c0);
    ld(y0 + 1, c1);
    ld(y0 + 2, ahead);
    f2 Lm1[5], Rm1[5], L0[5], R0[5], Fp[5], Fn[5];
    nf_recon<1, LIM>(P, cm2.v, cm1.v, c0.v, cf.half_dtdx, Lm1, Rm1);
    nf_recon<1, LIM>(P, cm1.v, c0.v, c1.v, cf.half_dtdx, L0, R0);
    nf_force4<1>(P, Rm1, L0, c4.dtdx, c4.dxdt, Fp);
    for (int y = y0; y < y1; y++) {
        // the next row is loaded one iteration ahead, so its latency overlaps this row's work
        c2 = ahead;
        if (y + 1 < y1) ld(y + 3, ahead);
        f2 L1[5], R1[5];
        nf_recon<1, LIM>(P, c0.v, c1.v, c2.v, cf.half_dtdx, L1, R1);
        nf_force4<1>(P, R0, L1, c4.dtdx, c4.dxdt, Fn);
        Cell2 nc;
        nf_update(c4.q_dtdx, c0.v, Fp, Fn, nc.v);
        st(y, nc);
        if (want_w) {
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
    return w;
}

// X sweep on one 64-cell row segment per warp: lane t holds the cells at positions s0 - 2 + 2t and
// s0 - 1 + 2t (s0 even).  x_pair_load fills the lane's pair (ghost positions mapped; positions
// more than two outside the row only feed the discarded halo work and are clamped to a valid
// ghost).
CG_D void x_pair_load(const Geom& G, const float* __restrict__ src, int row, int s0, Cell2& m) {
    const int lane = threadIdx.x & 31;
    const int n = G.nx;
    const int p0 = s0 - 2 + 2 * lane;
    const size_t rb = (size_t)row * G.pitch;
    if (p0 >= 0 && p0 + 1 < n) {
#pragma unroll
        for (int f = 0; f < 5; f++) m.v[f].v = *reinterpret_cast<const float2*>(src + f * G.fstride + rb + p0);
    } else {
        const int qa = ghost_index(min(p0, n + 1), n, G.bc), qb = ghost_index(min(p0 + 1, n + 1), n, G.bc);
#pragma unroll
        for (int f = 0; f < 5; f++) m.v[f].v = make_float2(src[f * G.fstride + rb + qa], src[f * G.fstride + rb + qb]);
    }
}

// The arithmetic of one X segment: neighbour cells, the next cell's left face state and the
// previous pair's right-face flux cross lanes by warp shuffles (no shared memory, no block
// barrier); nc receives the lane's two updated cells.  All 32 lanes call it together.
template <int LIM>
CG_D void x_pair_compute(const NewtonFastParams& P, const Cell2& m, const FastCoef& cf, Cell2& nc) {
    constexpr unsigned FULL = 0xffffffffu;
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
    const Force4Coef c4 = force4_coef(cf);
    nf_force4<0>(P, R, Rn, c4.dtdx, c4.dxdt, Fr);
#pragma unroll
    for (int f = 0; f < 5; f++) Fl[f].v = make_float2(__shfl_up_sync(FULL, Fr[f].v.y, 1), Fr[f].v.x);
    nf_update(c4.q_dtdx, m.v, Fl, Fr, nc.v);
}

// Lanes 1..30 store their two cells of the segment at s0 (60 per segment) and, when WS, return
// their wavespeed maximum (0 otherwise).  `full`: every lane's two cells lie inside the row (no
// per-lane bound checks).
template <bool WS>
CG_D float x_pair_store(const NewtonFastParams& P, int dims, const Geom& G, float* __restrict__ dst, int row, int s0,
                        const Cell2& nc, bool full) {
    const int lane = threadIdx.x & 31;
    const int n = G.nx;
    const int p0 = s0 - 2 + 2 * lane;
    float* d = dst + (size_t)row * G.pitch + p0;
    float w = 0.0f;
    if (lane < 1 || lane > 30) return w;
    if (full || p0 + 1 < n) {
        if (!full && p0 >= n) return w;
#pragma unroll
        for (int f = 0; f < 5; f++) *reinterpret_cast<float2*>(d + f * G.fstride) = nc.v[f].v;
        if (WS) {
            const f2 ws = nf_wavespeed(P, nc.v, dims);
            w = fmaxf(ws.v.x, ws.v.y);
        }
    } else if (p0 < n) {
#pragma unroll
        for (int f = 0; f < 5; f++) d[f * G.fstride] = nc.v[f].v.x;
        if (WS) w = fmaxf(nf_wavespeed(P, nc.v, dims).v.x, 0.0f);
    }
    return w;
}

// One X segment with run-time flags (the batched launch): compute when `act` (else store the
// cells unchanged), then store; returns the wavespeed maximum when want_w.
template <int LIM>
CG_D float x_pair_update(const NewtonFastParams& P, int dims, const Geom& G, float* __restrict__ dst, int row, int s0,
                         const Cell2& m, bool act, const FastCoef& cf, bool want_w) {
    Cell2 nc = m;
    if (act) x_pair_compute<LIM>(P, m, cf, nc);
    return want_w && act ? x_pair_store<true>(P, dims, G, dst, row, s0, nc, false)
                         : x_pair_store<false>(P, dims, G, dst, row, s0, nc, false);
}

// ---- single-grid kernels

// (Re)initialise one warp's R ring mbarriers; lane 0 works, the whole warp calls it.  A ring is
// drained between marches (every copy it issued has been waited for), so its barriers can be
// invalidated and initialised again: each march then starts at slot 0, phase 0, whose fixed
// slot and parity sequence compiles into cheaper code than a ring state carried in registers
// (measured 3 % on the 4096^2 Y sweep).
template <int R>
CG_D void ring_init(unsigned long long* bar, bool reinit) {
    if ((threadIdx.x & 31) == 0) {
        for (int q = 0; q < R; q++) {
            if (reinit) mbar_inval(&bar[q]);
            mbar_init(&bar[q], 1);
        }
        mbar_init_fence();
    }
    __syncwarp();
}

// Y march of one warp over rows [y0, y1) of the 64 columns from jw (two per lane), the rows
// arriving through the warp's ring of R row slots in shared memory (five field rows of 64 floats
// each, one mbarrier per slot, freshly initialised) by cp.async.bulk: lanes 0-4 copy one field
// each, up to R rows ahead of the row being consumed, so the loads overlap several rows of work
// where a register prefetch covers one.  The arithmetic is y_pair_march's.  All 32 lanes call it
// together, with jw < G.nx.  Returns the lane's wavespeed maximum over its updated cells when
// want_w.  A wait that runs out (about a second) makes `ok` false (warp-uniform); the warp then
// waits, again bounded, for its rows still in flight and returns.  On success the ring is drained.
template <int LIM, int R, int TM = 0>
CG_D float y_ring_march(const NewtonFastParams& P, int dims, const Geom& G, const float* __restrict__ src,
                        float* __restrict__ dst, int jw, int y0, int y1, const FastCoef cf, bool want_w,
                        float (*ring)[5][64], unsigned long long* bar, bool& ok, const CUtensorMap* tm = nullptr) {
    static_assert(R >= 5 && (R & (R - 1)) == 0, "a power of two above the four prologue rows");
    constexpr unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int j = jw + 2 * lane;
    const bool live = j < G.nx, two = j + 1 < G.nx;
    const Force4Coef c4 = force4_coef(cf);
    const uint32_t bytes = ((uint32_t)min(64, G.nx - jw) * 4u + 15u) & ~15u;  // within the padded pitch
    const int ylo = y0 - 2, yhi = y1 + 1;  // rows read
    // Row r of the ring lives in slot (r - ylo) mod R; the slot's k-th use completes phase k mod 2.
    // TM = 1 (TM = 2: when tm is not null): lane 0 copies the row's five fields as one box of the
    // tensor map tm; otherwise lanes 0-4 each copy one field (lanes 5+ hold a valid pointer they
    // never use).
    const float* fsrc = src + (size_t)min(lane, 4) * G.fstride + jw;
    int inext = ylo;  // warp-uniform: next row to issue
    auto issue_one = [&]() {
        const int r = inext, q = (r - ylo) & (R - 1);
        if (TM == 1 || (TM == 2 && tm)) {  // one copy of the row's five 64-column runs (columns past nx arrive as zeros)
            if (lane == 0) {
                mbar_expect_tx(&bar[q], 5 * 64 * 4);
                tma_load_3d(ring[q], tm, jw, ghost_index(r, G.ny, G.bc), 0, &bar[q]);
            }
        } else {
            if (lane == 0) mbar_expect_tx(&bar[q], 5 * bytes);
            __syncwarp();
            if (lane < 5) bulk_load(ring[q][lane], fsrc + (size_t)ghost_index(r, G.ny, G.bc) * G.pitch, bytes, &bar[q]);
        }
        ++inext;
    };
    for (int k = 0; k < R && inext <= yhi; k++) issue_one();
    bool mine = true;
    int tq = 0;         // slot of the next row to take
    uint32_t tpar = 0;  // its phase parity
    auto take = [&](Cell2& c) {
        mine = mine && mbar_wait(&bar[tq], tpar);
#pragma unroll
        for (int f = 0; f < 5; f++) {
            const float2 v = *reinterpret_cast<const float2*>(&ring[tq][f][2 * lane]);
            c.v[f].v = make_float2(v.x, two ? v.y : v.x);  // a lone last column runs in both lanes
        }
        if (++tq == R) {
            tq = 0;
            tpar ^= 1u;
        }
    };
    Cell2 cm2, cm1, c0, c1, c2;
    take(cm2);
    take(cm1);
    take(c0);
    take(c1);
    ok = __all_sync(FULL, mine);
    __syncwarp();  // every lane's reads of the freed slots are ordered before their refills
    float w = 0.0f;
    int consumed = ylo - 1;  // warp-uniform: last row every lane has copied out
    if (ok) {
        consumed = ylo + 3;
        for (int k = 0; k < 4 && inext <= yhi; k++) issue_one();
        f2 Lm1[5], Rm1[5], L0[5], R0[5], Fp[5], Fn[5];
        nf_recon<1, LIM>(P, cm2.v, cm1.v, c0.v, cf.half_dtdx, Lm1, Rm1);
        nf_recon<1, LIM>(P, cm1.v, c0.v, c1.v, cf.half_dtdx, L0, R0);
        nf_force4<1>(P, Rm1, L0, c4.dtdx, c4.dxdt, Fp);
        for (int y = y0; y < y1; y++) {
            take(c2);
            ok = __all_sync(FULL, mine);
            if (!ok) break;
            __syncwarp();
            consumed = y + 2;
            if (inext <= yhi) issue_one();
            f2 L1[5], R1[5];
            nf_recon<1, LIM>(P, c0.v, c1.v, c2.v, cf.half_dtdx, L1, R1);
            nf_force4<1>(P, R0, L1, c4.dtdx, c4.dxdt, Fn);
            Cell2 nc;
            nf_update(c4.q_dtdx, c0.v, Fp, Fn, nc.v);
            if (live) {
                const size_t b = (size_t)y * G.pitch + j;
#pragma unroll
                for (int f = 0; f < 5; f++) {
                    float* o = dst + f * G.fstride + b;
                    if (two) *reinterpret_cast<float2*>(o) = nc.v[f].v;
                    else *o = nc.v[f].v.x;
                }
                if (want_w) {
                    const f2 ws = nf_wavespeed(P, nc.v, dims);
                    w = fmaxf(w, fmaxf(ws.v.x, ws.v.y));  // a lone column's lanes are equal
                }
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
    if (!ok) {  // warp-uniform: rows consumed + 1 .. inext - 1 may still be in flight
        if (lane == 0)
            for (int r = consumed + 1; r < inext; r++)
                mbar_wait(&bar[(r - ylo) & (R - 1)], (uint32_t)((r - ylo) / R) & 1u, 100000000LL);
        __syncwarp();
    }
    return w;
}

// Y sweep with the rows staged in shared memory by bulk copies (y_ring_march; TM: one copy per row
// through the tensor map `tm` of the source's fields).  Block row b covers grid rows b seg ..
// (b + 1) seg - 1; each warp owns 64 columns and its own ring, never waits for the other warps (no
// block barrier after the set-up) and reduces its own CFL maximum.  A ring wait that runs out sets
// ST_TIMEOUT in the status word.
template <int LIM, int NT, int R, int MINB, bool TM>
__global__ void __launch_bounds__(NT, MINB) sweep_y_ring_kernel(NewtonFastParams P, int dims, Geom G,
                                                          const float* __restrict__ src, float* __restrict__ dst,
                                                          DtSrc ds, SweepOut out, int seg,
                                                          const __grid_constant__ CUtensorMap tm) {
    static_assert(NT % 32 == 0, "whole warps");
    constexpr int NWP = NT / 32;
    __shared__ __align__(128) float ring[NWP][R][5][64];
    __shared__ __align__(8) unsigned long long bar[NWP][R];
    __shared__ FastCoef s_coef;
    __shared__ int s_act;
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    const int jw = (blockIdx.x * NWP + wp) * 64;  // the warp's first column
    const int y0 = blockIdx.y * seg, y1 = min(y0 + seg, G.ny);
    if (threadIdx.x == 0) {
        double dt;
        s_act = ds.get(dt);
        if (s_act) s_coef = ds.fast_coef();
        for (int w = 0; w < NWP; w++)
            for (int q = 0; q < R; q++) mbar_init(&bar[w][q], 1);
        mbar_init_fence();
    }
    __syncthreads();
    if (jw >= G.nx) return;  // warp-uniform: no column of this warp exists
    if (!s_act) {            // inactive step: keep the ping-pong buffers consistent
        if (jw + 2 * lane < G.nx) y_pair_march<LIM>(P, dims, G, src, dst, jw + 2 * lane, y0, y1, false, s_coef, false);
        return;
    }
    bool ok = true;
    const FastCoef cf = s_coef;  // in registers: the ring's waits would make every use re-read shared memory
    // the reduction stays a run-time choice here: the compile-time form measured 3 % slower
    unsigned long long* wslot = out.slot();
    float w = y_ring_march<LIM, R, TM ? 1 : 0>(P, dims, G, src, dst, jw, y0, y1, cf, wslot != nullptr, ring[wp], bar[wp], ok,
                                       &tm);
    if (!ok) {
        if (lane == 0 && out.status) atomicOr(out.status, ST_TIMEOUT);
        return;
    }
    if (wslot) {
        w = warp_max(w);
        if (lane == 0) atomic_max_nonneg(wslot, (double)w);
    }
}

// X sweep with each warp's segments staged in shared memory by bulk copies: a one-warp block
// takes SEGS consecutive 60-cell segments of its row and, at its start, copies every segment whose
// 64-cell window lies inside the row (cells s0 - 4 .. s0 + 63, a 16-byte aligned run of 272 bytes
// per field) into its own slot, so all of them are in flight while the first is computed (TM: the
// five fields' windows as one box of the tensor map `tm`, one copy per segment); the row's first
// segment and its last ones (whose windows reach ghost cells) load through x_pair_load.  No registers hold a prefetched segment.  A wait that runs out (about a second)
// sets ST_TIMEOUT; the warp then waits, again bounded, for its copies still in flight and leaves.
template <int LIM, int SEGS, int MINB, bool WS, bool TM>
__global__ void __launch_bounds__(32, MINB) sweep_x_ring_kernel(NewtonFastParams P, int dims, Geom G,
                                                               const float* __restrict__ src, float* __restrict__ dst,
                                                               DtSrc ds, SweepOut out,
                                                               const __grid_constant__ CUtensorMap tm) {
    constexpr int TSW = 60, W = 68;
    constexpr int SLOT = (5 * W + 31) / 32 * 32;  // a slot holds fields 0-4 at f W; 128-byte aligned slots
    __shared__ __align__(128) float xr[SEGS][SLOT];
    __shared__ __align__(8) unsigned long long xb[SEGS];
    __shared__ FastCoef s_coef;
    __shared__ int s_act;
    const int lane = threadIdx.x;
    if (lane == 0) {
        double dt;
        s_act = ds.get(dt);
        if (s_act) s_coef = ds.fast_coef();
        for (int q = 0; q < SEGS; q++) mbar_init(&xb[q], 1);
        mbar_init_fence();
    }
    __syncthreads();
    const int n = G.nx, row = blockIdx.y;
    const int k0 = blockIdx.x * SEGS;
    const int kn = min(SEGS, (n + TSW - 1) / TSW - k0);  // segments of this warp (k0 < segments per row)
    if (!s_act) {  // inactive step: keep the ping-pong buffers consistent
        for (int i = 0; i < kn; i++) {
            Cell2 m;
            x_pair_load(G, src, row, (k0 + i) * TSW, m);
            x_pair_store<false>(P, dims, G, dst, row, (k0 + i) * TSW, m, false);
        }
        return;
    }
    // segment k's window s0 - 2 .. s0 + 61 lies inside the row and its copy s0 - 4 .. s0 + 63 too
    auto inside = [&](int k) { return k >= 1 && k * TSW + 64 <= n; };
    const size_t rb = (size_t)row * G.pitch;
    for (int i = 0; i < kn; i++) {
        if (!inside(k0 + i)) continue;
        if (TM) {  // the five fields' windows as one box
            if (lane == 0) {
                mbar_expect_tx(&xb[i], 5 * W * 4);
                tma_load_3d(xr[i], &tm, (k0 + i) * TSW - 4, row, 0, &xb[i]);
            }
        } else {
            if (lane == 0) mbar_expect_tx(&xb[i], 5 * W * 4);
            __syncwarp();
            if (lane < 5) bulk_load(&xr[i][lane * W], src + (size_t)lane * G.fstride + rb + (k0 + i) * TSW - 4, W * 4, &xb[i]);
        }
    }
    const FastCoef cf = s_coef;
    float w = 0.0f;
    for (int i = 0; i < kn; i++) {
        const int s0 = (k0 + i) * TSW;
        const bool in = inside(k0 + i);
        Cell2 m;
        if (in) {
            if (!__all_sync(0xffffffffu, mbar_wait(&xb[i], 0))) {
                if (lane == 0) {
                    if (out.status) atomicOr(out.status, ST_TIMEOUT);
                    for (int q = i; q < kn; q++)
                        if (inside(k0 + q)) mbar_wait(&xb[q], 0, 100000000LL);
                }
                __syncwarp();
                return;
            }
#pragma unroll
            for (int f = 0; f < 5; f++) m.v[f].v = *reinterpret_cast<const float2*>(&xr[i][f * W + 2 + 2 * lane]);
        } else {
            x_pair_load(G, src, row, s0, m);
        }
        Cell2 nc;
        x_pair_compute<LIM>(P, m, cf, nc);
        w = fmaxf(w, x_pair_store<WS>(P, dims, G, dst, row, s0, nc, in));
    }
    if (WS) {
        w = warp_max(w);
        if (lane == 0) atomic_max_nonneg(out.slot(), (double)w);
    }
}

}  // namespace cg
