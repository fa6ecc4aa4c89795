// Hand-written adjoint (vector-Jacobian product) of one Newtonian SLIC sweep.
//
// Forward map of a sweep along a line of n cells (conserved variables U, dt and dx fixed;
// Solvers/EulerSecondOrderSolver.cpp:3-100, Solvers/EulerSolvers.cpp:174-223,
// Solvers/EulerFirstOrderSolver.cpp:3-101, Solvers/SlopeLimiters.cpp:3-147):
//   slope_i  = xi(r_i) * (a (U_i - U_{i-1}) + b (U_{i+1} - U_i)),  a,b = (1 +- w)/2,
//              r_i = num/den of the two differences, each replaced by +1e-5 when |.| < 1e-5
//   UL_i, UR_i = U_i -+ slope_i / 2;   e_i = (dt/dx)/2 (F(UL_i) - F(UR_i))
//   A_i = UL_i + e_i (left-face state),  B_i = UR_i + e_i (right-face state)
//   F_{j+1/2} = FORCE(B_j, A_{j+1}) = ((LF + F(U*)) / 2 with LF = (F(L)+F(R))/2 + (dx/dt)(L-R)/2,
//              U* = (L+R)/2 + (dt/dx)(F(L)-F(R))/2
//   U'_i = U_i + (dt/dx) (F_{i-1/2} - F_{i+1/2})
// Given the adjoint of the output, Ubar', the adjoint of the input is
//   Ubar_i = Ubar'_i + sum over the cells whose half-step stencil holds i of their evolve VJP,
// where the face adjoints Fbar_{j+1/2} = (dt/dx)(Ubar'_{j+1} - Ubar'_j) are pulled back through
// FORCE to (Bbar_j, Abar_{j+1}) and then through each cell's half-step evolution.  Ghost cells
// (transmissive mirror or periodic wrap) pass their adjoint to the interior cell they copy.
// The limiter is differentiated piecewise (its derivative on the branch the forward takes; the
// clamped differences carry no derivative), as a dual-number evaluation of the same code would.
//
// Line tiles: P positions along the sweep axis (TS = P - 8 updated cells plus a 4-cell halo on each
// side) times W lines; one thread per position, five barrier-separated phases in shared memory:
//   0 load state and Ubar'   1 half-step evolution   2 FORCE reverse per face
//   3 half-step reverse per cell   4 gather per updated cell.
#pragma once
#include "device_common.cuh"
#include "sweep_kernels.cuh"

namespace cg {

// Reciprocal: approximate (about 1 ulp) in FP32, where the derivative does not need IEEE division;
// exact in FP64.
CG_D float adj_rcp(float x) { return __fdividef(1.0f, x); }
CG_D double adj_rcp(double x) { return 1.0 / x; }

// Newtonian flux along axis AX of a conserved state, and its transposed Jacobian.
template <class T>
struct AdjFlux {
    T g1;  // gamma - 1
    template <int AX>
    CG_D void flux(const T* u, T* f) const {
        const T inv = adj_rcp(u[0]);
        const T vn = u[1 + AX] * inv;
        const T p = g1 * (u[4] - T(0.5) * ((u[1] * u[1] + u[2] * u[2]) + u[3] * u[3]) * inv);
        f[0] = u[1 + AX];
        f[1] = u[1] * vn;
        f[2] = u[2] * vn;
        f[3] = u[3] * vn;
        f[1 + AX] = f[1 + AX] + p;
        f[4] = (u[4] + p) * vn;
    }
    // ub += (dF/du)^T gb
    template <int AX>
    CG_D void vjp(const T* u, const T* gb, T* ub) const {
        const T inv = adj_rcp(u[0]);
        const T v0 = u[1] * inv, v1 = u[2] * inv, v2 = u[3] * inv;
        const T vn = AX == 0 ? v0 : v1;
        const T vv = (v0 * v0 + v1 * v1) + v2 * v2;
        const T p = g1 * (u[4] - T(0.5) * u[0] * vv);
        const T pb = gb[1 + AX] + gb[4] * vn;                                         // from F_n and F_E
        const T vnb = ((gb[1] * u[1] + gb[2] * u[2]) + gb[3] * u[3]) + gb[4] * (u[4] + p);  // d/dv_n
        const T gp = g1 * pb;
        ub[0] += gp * T(0.5) * vv - vnb * vn * inv;
        ub[1] += gb[1] * vn - gp * v0;
        ub[2] += gb[2] * vn - gp * v1;
        ub[3] += gb[3] * vn - gp * v2;
        ub[1 + AX] += gb[0] + vnb * inv;
        ub[4] += gb[4] * vn + gp;
    }
};

// Limiter value and derivative d(xi)/dr on the branch the forward evaluation takes
// (Solvers/SlopeLimiters.cpp:8-69; min(a, b) picks b only when b < a).
template <class T, int LIM>
CG_D T limiter_d(T r, T w, T& d) {
    if (r < T(0)) { d = T(0); return T(0); }
    const T iden = adj_rcp((T(1) - w) + (T(1) + w) * r);
    const T xr = T(2) * iden;
    const T dxr = -T(2) * (T(1) + w) * iden * iden;
    if (LIM == 0) {  // SuperBee
        if (r < T(0.5)) { d = T(2); return T(2) * r; }
        if (r < T(1)) { d = T(0); return T(1); }
        T m = r;
        d = T(1);
        if (xr < m) { m = xr; d = dxr; }
        if (T(2) < m) { m = T(2); d = T(0); }
        return m;
    } else if (LIM == 1) {  // van Leer
        const T iop = adj_rcp(T(1) + r);
        const T vl = T(2) * r * iop;
        if (xr < vl) { d = dxr; return xr; }
        d = T(2) * iop * iop;
        return vl;
    }
    // MinBee
    if (r < T(1)) { d = T(1); return r; }
    if (xr < T(1)) { d = dxr; return xr; }
    d = T(0);
    return T(1);
}

// Half-step evolution of one cell: A (left-face) and B (right-face) states.
template <class T, int AX, int LIM>
CG_D void adj_evolve(const AdjFlux<T>& F, const T* ul, const T* uc, const T* ur, T w, T hs, T* A, T* B) {
    const T ca = T(0.5) * (T(1) + w), cb = T(0.5) * (T(1) - w);
    T UL[5], UR[5];
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const T dl = uc[k] - ul[k], dr = ur[k] - uc[k];
        const T s = ca * dl + cb * dr;
        const T num = fabs(dl) < T(1e-5) ? T(1e-5) : dl;
        const T den = fabs(dr) < T(1e-5) ? T(1e-5) : dr;
        T dxi;
        const T sl = s * limiter_d<T, LIM>(num * adj_rcp(den), w, dxi);
        UL[k] = uc[k] - T(0.5) * sl;
        UR[k] = uc[k] + T(0.5) * sl;
    }
    T FL[5], FR[5];
    F.template flux<AX>(UL, FL);
    F.template flux<AX>(UR, FR);
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const T e = hs * (FL[k] - FR[k]);
        A[k] = UL[k] + e;
        B[k] = UR[k] + e;
    }
}

// Reverse of adj_evolve: given Abar, Bbar, the contributions to the three stencil cells.
template <class T, int AX, int LIM>
CG_D void adj_evolve_vjp(const AdjFlux<T>& F, const T* ul, const T* uc, const T* ur, T w, T hs, const T* Ab,
                         const T* Bb, T* gl, T* gc, T* gr) {
    const T ca = T(0.5) * (T(1) + w), cb = T(0.5) * (T(1) - w);
    T UL[5], UR[5], sv[5], xi[5], dxi[5], r[5], iden[5];
    bool cn[5], cd[5];
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const T dl = uc[k] - ul[k], dr = ur[k] - uc[k];
        sv[k] = ca * dl + cb * dr;
        cn[k] = fabs(dl) < T(1e-5);
        cd[k] = fabs(dr) < T(1e-5);
        const T num = cn[k] ? T(1e-5) : dl;
        iden[k] = adj_rcp(cd[k] ? T(1e-5) : dr);
        r[k] = num * iden[k];
        xi[k] = limiter_d<T, LIM>(r[k], w, dxi[k]);
        const T sl = sv[k] * xi[k];
        UL[k] = uc[k] - T(0.5) * sl;
        UR[k] = uc[k] + T(0.5) * sl;
    }
    T ULb[5], URb[5], FLb[5], FRb[5];
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const T eb = Ab[k] + Bb[k];
        ULb[k] = Ab[k];
        URb[k] = Bb[k];
        FLb[k] = hs * eb;
        FRb[k] = -(hs * eb);
    }
    F.template vjp<AX>(UL, FLb, ULb);
    F.template vjp<AX>(UR, FRb, URb);
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const T slb = T(0.5) * (URb[k] - ULb[k]);
        const T xib = slb * sv[k];
        const T sb = slb * xi[k];
        const T rb = xib * dxi[k];
        const T dlb = ca * sb + (cn[k] ? T(0) : rb * iden[k]);
        const T drb = cb * sb - (cd[k] ? T(0) : rb * r[k] * iden[k]);
        gl[k] = -dlb;
        gc[k] = (ULb[k] + URb[k]) + (dlb - drb);
        gr[k] = drb;
    }
}

// Reverse of the FORCE flux of (L, R): given Fbar, Lbar and Rbar.
template <class T, int AX>
CG_D void adj_force_vjp(const AdjFlux<T>& F, const T* L, const T* R, T c, T d, const T* Fb, T* Lb, T* Rb) {
    T fL[5], fR[5], us[5];
    F.template flux<AX>(L, fL);
    F.template flux<AX>(R, fR);
#pragma unroll
    for (int k = 0; k < 5; k++) us[k] = T(0.5) * ((L[k] + R[k]) + d * (fL[k] - fR[k]));
    T usb[5] = {T(0), T(0), T(0), T(0), T(0)}, fsb[5];
#pragma unroll
    for (int k = 0; k < 5; k++) fsb[k] = T(0.5) * Fb[k];
    F.template vjp<AX>(us, fsb, usb);
    T fLb[5], fRb[5];
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const T lfb = T(0.5) * Fb[k];
        Lb[k] = T(0.5) * usb[k] + T(0.5) * c * lfb;
        Rb[k] = T(0.5) * usb[k] - T(0.5) * c * lfb;
        fLb[k] = T(0.5) * d * usb[k] + T(0.5) * lfb;
        fRb[k] = T(0.5) * lfb - T(0.5) * d * usb[k];
    }
    F.template vjp<AX>(L, fLb, Lb);
    F.template vjp<AX>(R, fRb, Rb);
}

// Coefficients of one sweep, formed on the host in both precisions (an FP64 divide per thread
// would dominate the FP32 kernel: GB300's FP64 rate is 1/64 of FP32).
template <class T>
struct AdjCoef {
    T g1, gam, w, d, c, hs;  // gamma - 1, gamma, bias, dt/dx, dx/dt, dt/(2 dx)
};
struct AdjSweepParams {
    Geom G;
    double dx, dt, bias, gamma;
    AdjCoef<float> cf;
    AdjCoef<double> cd;
    const void* state;     // sweep input in storage precision (FP64 primitives or FP32 conserved)
    const void* ubar_out;  // adjoint of the sweep output (T, conserved SoA, same layout)
    void* ubar_in;         // adjoint of the sweep input (written)
};

// Transmissive mirror (exact for up to two cells out) or periodic wrap, clamped into the line for
// the positions further out that only feed discarded halo work.
CG_D int adj_map(int i, int n, bool per) {
    if (per) {
        if (i >= 0 && i < n) return i;
        if (i < 0 && i >= -n) return i + n;
        if (i >= n && i < 2 * n) return i - n;
        return ((i % n) + n) % n;
    }
    int m = i < 0 ? -1 - i : (i >= n ? 2 * n - 1 - i : i);
    return m < 0 ? 0 : (m >= n ? n - 1 : m);
}

template <class T, class S, bool PRIM, int AX, int LIM, int P, int W>
__global__ void __launch_bounds__(P * W, (sizeof(T) == 4 ? 3 : 1)) adjoint_sweep_kernel(AdjSweepParams a) {
    constexpr int TS = P - 8;
    constexpr int NW = P * W;
    extern __shared__ __align__(16) unsigned char adj_smem[];
    T* sA = (T*)adj_smem;   // [5]  state
    T* sB = sA + 5 * NW;    // [5]  Ubar' (phase 0-2), then the contribution to the right neighbour
    T* sC = sB + 5 * NW;    // [10] A,B evolved states (1-2), then contributions to self and left neighbour
    T* sD = sC + 10 * NW;   // [10] Abar of the right state, Bbar of the left state per face
    const Geom& G = a.G;
    const int along = AX == 0 ? threadIdx.x : threadIdx.y;
    const int across = AX == 0 ? threadIdx.y : threadIdx.x;
    const int n = AX == 0 ? G.nx : G.ny;
    const int nl = AX == 0 ? G.ny : G.nx;
    const int line = (AX == 0 ? blockIdx.y : blockIdx.x) * W + across;
    const int s0 = (AX == 0 ? blockIdx.x : blockIdx.y) * TS;
    const int k = s0 - 4 + along;
    const bool lok = line < nl;
    const bool per = G.bc == 1;
    // shared index of (across, position): positions contiguous for X, lines contiguous for Y
    auto si = [&](int pos) { return AX == 0 ? across * P + pos : pos * W + across; };
    auto gi = [&](int pos) -> size_t {
        return AX == 0 ? (size_t)line * G.pitch + pos : (size_t)pos * G.pitch + line;
    };
    AdjCoef<T> K;
    if constexpr (sizeof(T) == 4) K = a.cf;
    else K = a.cd;
    const AdjFlux<T> F{K.g1};
    const T w = K.w, d = K.d, c = K.c, hs = K.hs;
    const S* st = (const S*)a.state;
    const T* ubo = (const T*)a.ubar_out;
    const int me = si(along);

    // ---- 0: state and Ubar' at this position
    T ub_own[5];
    {
        T u[5] = {T(1), T(0), T(0), T(0), T(1)};
        T b[5] = {T(0), T(0), T(0), T(0), T(0)};
        if (lok) {
            const size_t q = gi(adj_map(k, n, per));
            T v[5];
#pragma unroll
            for (int f = 0; f < 5; f++) v[f] = T(st[f * G.fstride + q]);
            if (PRIM) {  // Euler/EulerStateVector.cpp:55-66
                u[0] = v[0];
                u[1] = v[0] * v[1];
                u[2] = v[0] * v[2];
                u[3] = v[0] * v[3];
                u[4] = v[0] * (T(0.5) * ((v[1] * v[1] + v[2] * v[2]) + v[3] * v[3]) + v[4] / (K.g1 * v[0]));
            } else {
#pragma unroll
                for (int f = 0; f < 5; f++) u[f] = v[f];
            }
            if (per || (k >= 0 && k < n)) {
#pragma unroll
                for (int f = 0; f < 5; f++) b[f] = ubo[f * G.fstride + q];
            }
        }
#pragma unroll
        for (int f = 0; f < 5; f++) {
            sA[f * NW + me] = u[f];
            sB[f * NW + me] = b[f];
            ub_own[f] = b[f];
        }
    }
    __syncthreads();
    auto ld = [&](const T* arr, int pos, T* out) {
        const int x = si(pos);
#pragma unroll
        for (int f = 0; f < 5; f++) out[f] = arr[f * NW + x];
    };
    // ---- 1: half-step evolution of every cell with both neighbours in the tile
    if (lok && along >= 1 && along < P - 1) {
        T ul[5], uc[5], ur[5], A[5], B[5];
        ld(sA, along - 1, ul);
        ld(sA, along, uc);
        ld(sA, along + 1, ur);
        adj_evolve<T, AX, LIM>(F, ul, uc, ur, w, hs, A, B);
#pragma unroll
        for (int f = 0; f < 5; f++) {
            sC[f * NW + me] = A[f];
            sC[(5 + f) * NW + me] = B[f];
        }
    }
    __syncthreads();
    // ---- 2: FORCE reverse at the face between this cell (k) and the next (k + 1)
    if (along >= 1 && along < P - 2) {
        T Lb[5] = {T(0), T(0), T(0), T(0), T(0)}, Rb[5] = {T(0), T(0), T(0), T(0), T(0)};
        if (lok && (per || (k >= -1 && k <= n - 1))) {
            T L[5], R[5], Fb[5];
            const int nx1 = si(along + 1);
#pragma unroll
            for (int f = 0; f < 5; f++) {
                L[f] = sC[(5 + f) * NW + me];
                R[f] = sC[f * NW + nx1];
                Fb[f] = d * (sB[f * NW + nx1] - sB[f * NW + me]);
            }
            adj_force_vjp<T, AX>(F, L, R, c, d, Fb, Lb, Rb);
        }
#pragma unroll
        for (int f = 0; f < 5; f++) {
            sD[f * NW + me] = Lb[f];       // adjoint of B_k
            sD[(5 + f) * NW + me] = Rb[f]; // adjoint of A_{k+1}
        }
    }
    __syncthreads();
    // ---- 3: half-step reverse of this cell; neither sB nor sC is read in this phase
    if (along >= 2 && along < P - 2) {
        T gl[5] = {T(0), T(0), T(0), T(0), T(0)}, gc[5] = {T(0), T(0), T(0), T(0), T(0)},
          gr[5] = {T(0), T(0), T(0), T(0), T(0)};
        if (lok && (per || (k >= -1 && k <= n))) {
            T ul[5], uc[5], ur[5], Ab[5], Bb[5];
            ld(sA, along - 1, ul);
            ld(sA, along, uc);
            ld(sA, along + 1, ur);
            const int pv = si(along - 1);
#pragma unroll
            for (int f = 0; f < 5; f++) {
                Bb[f] = sD[f * NW + me];
                Ab[f] = sD[(5 + f) * NW + pv];
            }
            adj_evolve_vjp<T, AX, LIM>(F, ul, uc, ur, w, hs, Ab, Bb, gl, gc, gr);
        }
#pragma unroll
        for (int f = 0; f < 5; f++) {
            sC[f * NW + me] = gc[f];
            sC[(5 + f) * NW + me] = gl[f];
            sB[f * NW + me] = gr[f];
        }
    }
    __syncthreads();
    // ---- 4: gather for the updated cells
    if (lok && along >= 4 && along < 4 + TS && k < n) {
        T acc[5];
#pragma unroll
        for (int f = 0; f < 5; f++) acc[f] = ub_own[f];
        if (k >= 2 && k <= n - 3) {
            // interior (n >= 5): the right neighbour of k - 1, k itself, the left neighbour of k + 1
            const int xl = si(along - 1), xr = si(along + 1);
#pragma unroll
            for (int f = 0; f < 5; f++) acc[f] += (sB[f * NW + xl] + sC[f * NW + me]) + sC[(5 + f) * NW + xr];
        } else
#pragma unroll
        for (int dd = -2; dd <= 2; dd++) {
            const int i = k + dd;
            if (!per && (i < -1 || i > n)) continue;
            if (per && dd - n >= -2) continue;  // same physical cell as an earlier dd (n <= 4)
            const int x = si(along + dd);
#pragma unroll
            for (int q = -1; q <= 1; q++) {
                const int tgt = per ? ((i + q) % n + n) % n : (i + q < 0 ? -1 - (i + q) : (i + q >= n ? 2 * n - 1 - (i + q) : i + q));
                if (tgt != k) continue;
                const T* src = q == -1 ? sC + 5 * NW : (q == 0 ? sC : sB);
#pragma unroll
                for (int f = 0; f < 5; f++) acc[f] += src[f * NW + x];
            }
        }
        T* ubi = (T*)a.ubar_in;
        const size_t q = gi(k);
#pragma unroll
        for (int f = 0; f < 5; f++) ubi[f * G.fstride + q] = acc[f];
    }
}

// Loss L = 1/2 sum (rho - target)^2 over the grid, seed Ubar = (rho - target, 0, 0, 0, 0).
// One block per row; the row sums are added in row order by adjoint_loss_final_kernel.
template <class T, class S>
__global__ void __launch_bounds__(256) adjoint_loss_kernel(Geom G, const S* state, const double* target, T* ubar,
                                                           double* row_sums) {
    const int i = blockIdx.x;
    double acc = 0.0;
    for (int j = threadIdx.x; j < G.nx; j += 256) {
        const size_t q = (size_t)i * G.pitch + j;
        const double e = (double)state[q] - target[(size_t)i * G.nx + j];
        acc += 0.5 * e * e;
        ubar[q] = T(e);
#pragma unroll
        for (int f = 1; f < 5; f++) ubar[f * G.fstride + q] = T(0);
    }
    __shared__ double red[256];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) row_sums[i] = red[0];
}

static __global__ void __launch_bounds__(32) adjoint_loss_final_kernel(const double* row_sums, int n, double* loss) {
    if (threadIdx.x != 0) return;
    double s = 0.0;
    for (int i = 0; i < n; i++) s += row_sums[i];
    *loss = s;
}

// Gradient with respect to the initial primitives: Pbar = (dU/dP)^T Ubar at the initial state,
// written as AoS doubles (the layout of cosmos_grid_set_prim).
template <class T, class S, bool PRIM>
__global__ void adjoint_grad_kernel(Geom G, double gamma, const S* state, const T* ubar, double* grad) {
    const size_t ncell = (size_t)G.nx * G.ny;
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < ncell; c += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(c / G.nx), j = (int)(c % G.nx);
        const size_t q = (size_t)i * G.pitch + j;
        double v[5], u[5];
#pragma unroll
        for (int f = 0; f < 5; f++) {
            v[f] = (double)state[f * G.fstride + q];
            u[f] = (double)ubar[f * G.fstride + q];
        }
        double rho, vx, vy, vz;
        if (PRIM) {
            rho = v[0]; vx = v[1]; vy = v[2]; vz = v[3];
        } else {
            rho = v[0]; vx = v[1] / rho; vy = v[2] / rho; vz = v[3] / rho;
        }
        const double vv = vx * vx + vy * vy + vz * vz;
        double* o = grad + 5 * c;
        o[0] = u[0] + u[1] * vx + u[2] * vy + u[3] * vz + u[4] * 0.5 * vv;
        o[1] = rho * (u[1] + u[4] * vx);
        o[2] = rho * (u[2] + u[4] * vy);
        o[3] = rho * (u[3] + u[4] * vz);
        o[4] = u[4] / (gamma - 1.0);
    }
}

}  // namespace cg

namespace cg {

// Launch the sweep adjoint for one axis.  Tiles of 256 threads (three resident per SM in FP32): X lines of
// 256 positions (248 updated cells); Y lines of 64 positions (56 cells) x 4 adjacent columns.
template <class T, class S, bool PRIM, int AX, int LIM>
cudaError_t launch_adjoint_sweep_t(const AdjSweepParams& a, cudaStream_t st) {
    constexpr int P = AX == 0 ? 256 : 64;
    constexpr int W = AX == 0 ? 1 : 4;
    constexpr int TS = P - 8;
    const size_t smem = (size_t)30 * P * W * sizeof(T);
    auto kern = adjoint_sweep_kernel<T, S, PRIM, AX, LIM, P, W>;
    static bool attr_set = false;  // per instantiation; the attribute is per function and device-independent here
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    const Geom& G = a.G;
    dim3 block = AX == 0 ? dim3(P, W) : dim3(W, P);
    dim3 grid = AX == 0 ? dim3((G.nx + TS - 1) / TS, (G.ny + W - 1) / W) : dim3((G.nx + W - 1) / W, (G.ny + TS - 1) / TS);
    kern<<<grid, block, smem, st>>>(a);
    return cudaGetLastError();
}

template <class T, class S, bool PRIM>
cudaError_t launch_adjoint_sweep_any(const AdjSweepParams& a, int lim, cudaStream_t st) {
    const int ax = a.G.axis;
    if (ax == 0) {
        if (lim == 0) return launch_adjoint_sweep_t<T, S, PRIM, 0, 0>(a, st);
        if (lim == 1) return launch_adjoint_sweep_t<T, S, PRIM, 0, 1>(a, st);
        return launch_adjoint_sweep_t<T, S, PRIM, 0, 2>(a, st);
    }
    if (lim == 0) return launch_adjoint_sweep_t<T, S, PRIM, 1, 0>(a, st);
    if (lim == 1) return launch_adjoint_sweep_t<T, S, PRIM, 1, 1>(a, st);
    return launch_adjoint_sweep_t<T, S, PRIM, 1, 2>(a, st);
}

template <class T, class S, bool PRIM>
cudaError_t launch_adjoint_loss_t(const Geom& G, const void* state, const double* target, void* ubar, double* row_sums,
                                  double* loss, cudaStream_t st) {
    adjoint_loss_kernel<T, S><<<G.ny, 256, 0, st>>>(G, (const S*)state, target, (T*)ubar, row_sums);
    adjoint_loss_final_kernel<<<1, 32, 0, st>>>(row_sums, G.ny, loss);
    return cudaGetLastError();
}

template <class T, class S, bool PRIM>
cudaError_t launch_adjoint_grad_t(const Geom& G, double gamma, const void* state, const void* ubar, double* grad,
                                  cudaStream_t st) {
    const size_t ncell = (size_t)G.nx * G.ny;
    const int blocks = (int)std::min<size_t>((ncell + 255) / 256, 152 * 16);
    adjoint_grad_kernel<T, S, PRIM><<<blocks, 256, 0, st>>>(G, gamma, (const S*)state, (const T*)ubar, grad);
    return cudaGetLastError();
}

}  // namespace cg
