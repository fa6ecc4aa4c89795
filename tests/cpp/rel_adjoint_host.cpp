// Host build of the relativistic adjoints' cell functions (the bodies of rel_adjoint_sweep_kernel
// and rel_adjoint_rk_kernel) for the CPU tests.  AoS (ny, nx, 5) doubles in and out; in between a
// structure-of-arrays copy with the device grid's kind of padding (row pitch nx + 3, field stride
// ny * pitch + 5) whose padding holds NaN, so a read outside the cells it should touch shows up
// in the result.  system 1 = SR, 2 = black hole (bh = M, a, x, y, z; dims 1 or 2).
#include <cstddef>
#include <limits>
#include <vector>

#include "../../cosmos_gb300/csrc/adjoint_rel.cuh"

namespace {

// Runs `cell` over every cell of a padded structure-of-arrays copy of the AoS inputs.
template <class F>
int run_padded(int system, int dims, const double* state, const double* pbar_out, double* pbar_in, int ny, int nx,
               int axis, int bc, double gamma, const double* bh, double dx, double dt, double bias, int lim, F cell) {
    if (nx < 2 || ny < 1 || (axis == 1 && ny < 2)) return 1;
    const int pitch = nx + 3;
    const size_t fstride = (size_t)ny * pitch + 5;
    const double nan = std::numeric_limits<double>::quiet_NaN();
    std::vector<double> s(5 * fstride, nan), po(5 * fstride, nan), pi(5 * fstride, nan);
    for (int i = 0; i < ny; i++)
        for (int j = 0; j < nx; j++)
            for (int f = 0; f < 5; f++) {
                s[f * fstride + (size_t)i * pitch + j] = state[((size_t)i * nx + j) * 5 + f];
                po[f * fstride + (size_t)i * pitch + j] = pbar_out[((size_t)i * nx + j) * 5 + f];
            }
    cg::radj::Params P;
    P.system = system;
    P.dims = dims;
    P.nx = nx;
    P.ny = ny;
    P.pitch = pitch;
    P.periodic = bc == 1;
    P.fstride = fstride;
    P.gamma = gamma;
    for (int k = 0; k < 5; k++) P.bh[k] = bh ? bh[k] : 0.0;
    P.s = cg::radj::Step{dx, dt, bias, lim, axis};
    P.state = s.data();
    P.pbar_out = po.data();
    P.pbar_in = pi.data();
    for (size_t c = 0; c < (size_t)nx * ny; c++) cell(P, c);
    for (int i = 0; i < ny; i++)
        for (int j = 0; j < nx; j++)
            for (int f = 0; f < 5; f++) pbar_in[((size_t)i * nx + j) * 5 + f] = pi[f * fstride + (size_t)i * pitch + j];
    return 0;
}

}  // namespace

// One sweep's adjoint (the body of rel_adjoint_sweep_kernel).
extern "C" int rel_host_sweep_adjoint(int system, int dims, const double* state, const double* pbar_out,
                                      double* pbar_in, int ny, int nx, int axis, int bc, double gamma, const double* bh,
                                      double dx, double dt, double bias, int lim) {
    return run_padded(system, dims, state, pbar_out, pbar_in, ny, nx, axis, bc, gamma, bh, dx, dt, bias, lim,
                      [](const cg::radj::Params& P, size_t c) { cg::radj::cell_adjoint(P, c); });
}

// One black-hole RK source step's adjoint (the body of rel_adjoint_rk_kernel); transmissive.
extern "C" int rel_host_rk_adjoint(int dims, const double* state, const double* pbar_out, double* pbar_in, int ny,
                                   int nx, double gamma, const double* bh, double dx, double dt) {
    return run_padded(2, dims, state, pbar_out, pbar_in, ny, nx, 0, 0, gamma, bh, dx, dt, 0.0, 1,
                      [](const cg::radj::Params& P, size_t c) { cg::radj::rk_cell_adjoint(P, c); });
}
