// C ABI of the state-level functions: the reference's state-vector, equation-of-state, slope-limiter
// and black-hole eigenvalue functions for arrays of states, evaluated on the device by the
// reference-exact kernels (kernels_exact.cu, FP64, no contraction).  Host arrays in, host arrays out.
#include <cstring>
#include <string>

#include "capi_internal.h"

using namespace cg;

static_assert(COSMOS_STATE_CONS == kStateCons && COSMOS_STATE_PRIM == kStatePrim && COSMOS_STATE_FLUX_X == kStateFluxX &&
                  COSMOS_STATE_FLUX_Y == kStateFluxY && COSMOS_STATE_SOUND == kStateSound &&
                  COSMOS_STATE_INTERNAL_ENERGY == kStateInternalEnergy && COSMOS_STATE_TOTAL_ENERGY == kStateTotalEnergy &&
                  COSMOS_STATE_PRESSURE == kStatePressure && COSMOS_STATE_ENTHALPY == kStateEnthalpy &&
                  COSMOS_STATE_SOURCE == kStateSource && COSMOS_STATE_EIGENVALUES == kStateEigenvalues &&
                  COSMOS_STATE_GRADIENT_RATIO == kStateGradientRatio && COSMOS_STATE_LIMITER == kStateLimiter &&
                  COSMOS_STATE_SLOPE == kStateSlope,
              "state operation codes of the public header and the kernels differ");

namespace {

int sfail(int code, const std::string& msg) {
    set_error(msg.c_str());
    return code;
}
#define SCK(call)                                                                                    \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess) return sfail(COSMOS_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

}  // namespace

extern "C" {

int cosmos_state_width(int op, size_t* in_width, size_t* out_width) {
    size_t i = 5, o = 5;
    switch (op) {
        case COSMOS_STATE_CONS: case COSMOS_STATE_PRIM: case COSMOS_STATE_FLUX_X: case COSMOS_STATE_FLUX_Y:
        case COSMOS_STATE_SOURCE:
            break;
        case COSMOS_STATE_SOUND: case COSMOS_STATE_INTERNAL_ENERGY: case COSMOS_STATE_TOTAL_ENERGY:
        case COSMOS_STATE_PRESSURE: case COSMOS_STATE_ENTHALPY:
            o = 1;
            break;
        case COSMOS_STATE_EIGENVALUES: o = 9; break;
        case COSMOS_STATE_GRADIENT_RATIO: case COSMOS_STATE_LIMITER: i = 1; o = 1; break;
        case COSMOS_STATE_SLOPE: i = 15; break;
        default: return sfail(COSMOS_EINVAL, "unknown state operation " + std::to_string(op));
    }
    if (in_width) *in_width = i;
    if (out_width) *out_width = o;
    return COSMOS_OK;
}

int cosmos_state_eval(cosmos_ctx* ctx, const cosmos_params* p, int op, size_t n, const double* in, const double* xyz,
                      double bias, int limiter, double* out) {
    size_t wi = 0, wo = 0;
    int rc = cosmos_state_width(op, &wi, &wo);
    if (rc) return rc;
    if (!ctx || !p) return sfail(COSMOS_EINVAL, "null context or params");
    if (n == 0) return COSMOS_OK;
    if (!in || !out) return sfail(COSMOS_EINVAL, "null input or output array");
    const bool limiter_op = op == COSMOS_STATE_GRADIENT_RATIO || op == COSMOS_STATE_LIMITER || op == COSMOS_STATE_SLOPE;
    if (!limiter_op) {
        if (p->system < COSMOS_NEWTONIAN || p->system > COSMOS_GR) return sfail(COSMOS_EINVAL, "unknown system");
        if (!(p->gamma > 1.0)) return sfail(COSMOS_EINVAL, "gamma must exceed 1");
        const bool newton_only = op == COSMOS_STATE_INTERNAL_ENERGY || op == COSMOS_STATE_TOTAL_ENERGY ||
                                 op == COSMOS_STATE_PRESSURE;
        if (newton_only && p->system != COSMOS_NEWTONIAN)
            return sfail(COSMOS_EUNSUPPORTED, "internal energy, total energy and pressure belong to the Newtonian system");
        if (op == COSMOS_STATE_ENTHALPY && p->system == COSMOS_NEWTONIAN)
            return sfail(COSMOS_EUNSUPPORTED, "the specific enthalpy belongs to the relativistic systems");
        if ((op == COSMOS_STATE_SOURCE || op == COSMOS_STATE_EIGENVALUES) && p->system != COSMOS_GR)
            return sfail(COSMOS_EUNSUPPORTED, "source terms and eigenvalues belong to the black-hole system");
        if (p->system == COSMOS_GR && !xyz) return sfail(COSMOS_EINVAL, "black-hole states need coordinates");
        if (op == COSMOS_STATE_SOURCE && !(p->dx > 0.0)) return sfail(COSMOS_EINVAL, "source terms need dx > 0");
    }
    const bool coords = !limiter_op && p->system == COSMOS_GR;
    SCK(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const size_t bin = n * wi * sizeof(double), bout = n * wo * sizeof(double), bxyz = coords ? n * 3 * sizeof(double) : 0;
    char* d = nullptr;
    SCK(cudaMallocAsync((void**)&d, bin + bout + bxyz, st));
    SweepArgs s;
    memset(&s, 0, sizeof s);
    s.system = limiter_op ? COSMOS_NEWTONIAN : p->system;
    s.gamma = p->gamma;
    s.dx = p->dx;
    s.bh[0] = p->bh_mass; s.bh[1] = p->bh_spin; s.bh[2] = p->bh_x; s.bh[3] = p->bh_y; s.bh[4] = p->bh_z;
    s.stream = st;
    StateEvalArgs a;
    a.system = s.system;
    a.op = op;
    a.n = n;
    a.in = (const double*)d;
    a.out = (double*)(d + bin);
    a.xyz = coords ? (const double*)(d + bin + bout) : nullptr;
    a.in_stride = wi;
    a.out_stride = wo;
    a.gamma = p->gamma;
    a.bias = bias;
    a.lim = limiter;
    cudaError_t e = cudaMemcpyAsync(d, in, bin, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && coords) e = cudaMemcpyAsync(d + bin + bout, xyz, bxyz, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = launch_state_eval(s, a);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, d + bin, bout, cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(d, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return sfail(COSMOS_ECUDA, std::string("state evaluation: ") + cudaGetErrorString(e));
    return COSMOS_OK;
}

static_assert(COSMOS_IF_LAX_FRIEDRICHS == 0 && COSMOS_IF_EVOLUTION == 5 && COSMOS_IF_X_LAX_FRIEDRICHS_FLUX == 6 &&
                  COSMOS_IF_Y_FORCE_FLUX == 11 && COSMOS_IF_X_SLIC_FLUX == 12 && COSMOS_IF_EVOLVE_HALF_X == 14 &&
                  COSMOS_IF_EVOLVE_HALF_VECTOR_Y == 17 && COSMOS_IF_EVOLVE_FRACTION_X == 18 &&
                  COSMOS_IF_EVOLVE_FRACTION_VECTOR == 20 && COSMOS_IF_RK_CELL_2D == 22 && kIfaceOps == 23,
              "interface operation codes of the public header and the kernels differ");

static_assert(COSMOS_SPACETIME_WIDTH == kSpacetimeWidth && COSMOS_ST_EXCISED == kSpacetimeWidth - 1,
              "spacetime record layouts of the public header and the kernel differ");

int cosmos_spacetime_eval(cosmos_ctx* ctx, const cosmos_params* p, size_t n, const double* xyz, double* out) {
    if (!ctx || !p) return sfail(COSMOS_EINVAL, "null context or params");
    if (n == 0) return COSMOS_OK;
    if (!xyz || !out) return sfail(COSMOS_EINVAL, "null coordinate or output array");
    if (!(p->dx > 0.0)) return sfail(COSMOS_EINVAL, "the derivative spacing (params dx, the reference's cellSpacing) must be positive");
    SCK(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const size_t bq = n * 3 * sizeof(double), bo = n * kSpacetimeWidth * sizeof(double);
    char* d = nullptr;
    SCK(cudaMallocAsync((void**)&d, bq + bo, st));
    SweepArgs s;
    memset(&s, 0, sizeof s);
    s.system = COSMOS_GR;
    s.gamma = p->gamma > 1.0 ? p->gamma : 5.0 / 3.0;
    s.dx = p->dx;
    s.bh[0] = p->bh_mass; s.bh[1] = p->bh_spin; s.bh[2] = p->bh_x; s.bh[3] = p->bh_y; s.bh[4] = p->bh_z;
    s.stream = st;
    cudaError_t e = cudaMemcpyAsync(d, xyz, bq, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = launch_spacetime_eval(s, n, (const double*)d, (double*)(d + bq));
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, d + bq, bo, cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(d, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return sfail(COSMOS_ECUDA, std::string("spacetime evaluation: ") + cudaGetErrorString(e));
    return COSMOS_OK;
}

int cosmos_interface_width(int op, size_t* in_width, size_t* out_width) {
    if (op < 0 || op >= kIfaceOps) return sfail(COSMOS_EINVAL, "unknown interface operation " + std::to_string(op));
    if (in_width) *in_width = (size_t)kIfaceWidth[op];
    if (out_width) *out_width = 5;
    return COSMOS_OK;
}

int cosmos_interface_eval(cosmos_ctx* ctx, const cosmos_params* p, int op, size_t n, const double* in, const double* xyz,
                          double dt, double bias, int limiter, double frac, int side, double* out) {
    size_t wi = 0;
    int rc = cosmos_interface_width(op, &wi, nullptr);
    if (rc) return rc;
    if (!ctx || !p) return sfail(COSMOS_EINVAL, "null context or params");
    if (n == 0) return COSMOS_OK;
    if (!in || !out) return sfail(COSMOS_EINVAL, "null input or output array");
    if (p->system < COSMOS_NEWTONIAN || p->system > COSMOS_GR) return sfail(COSMOS_EINVAL, "unknown system");
    if (!(p->gamma > 1.0)) return sfail(COSMOS_EINVAL, "gamma must exceed 1");
    if (!(p->dx > 0.0) || !(dt > 0.0)) return sfail(COSMOS_EINVAL, "cellSpacing (params dx) and timeStep must be positive");
    if (op >= COSMOS_IF_EVOLVE_FRACTION_X && p->system != COSMOS_GR)
        return sfail(COSMOS_EUNSUPPORTED, "fractional evolutions and the forcing solver's cell update belong to the "
                                          "black-hole system");
    if ((op >= COSMOS_IF_EVOLVE_HALF_X && op <= COSMOS_IF_EVOLVE_HALF_VECTOR_Y) && side != 0 && side != 1)
        return sfail(COSMOS_EINVAL, "side must be 0 (left / top face) or 1 (right / bottom face)");
    const bool coords = p->system == COSMOS_GR && op >= COSMOS_IF_X_LAX_FRIEDRICHS_FLUX;
    if (coords && !xyz) return sfail(COSMOS_EINVAL, "black-hole functions need the coordinate arguments (xyz)");
    SCK(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const size_t bin = n * wi * sizeof(double), bout = n * 5 * sizeof(double), bxyz = coords ? n * 3 * sizeof(double) : 0;
    char* d = nullptr;
    SCK(cudaMallocAsync((void**)&d, bin + bout + bxyz, st));
    SweepArgs s;
    memset(&s, 0, sizeof s);
    s.system = p->system;
    s.gamma = p->gamma;
    s.dx = p->dx;
    s.bh[0] = p->bh_mass; s.bh[1] = p->bh_spin; s.bh[2] = p->bh_x; s.bh[3] = p->bh_y; s.bh[4] = p->bh_z;
    s.stream = st;
    IfaceArgs a;
    a.system = p->system;
    a.op = op;
    a.n = n;
    a.in = (const double*)d;
    a.out = (double*)(d + bin);
    a.xyz = coords ? (const double*)(d + bin + bout) : nullptr;
    a.dx = p->dx;
    a.dt = dt;
    a.bias = bias;
    a.frac = frac;
    a.lim = limiter;
    a.side = side;
    a.width = (int)wi;
    cudaError_t e = cudaMemcpyAsync(d, in, bin, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && coords) e = cudaMemcpyAsync(d + bin + bout, xyz, bxyz, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = launch_interface_eval(s, a);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, d + bin, bout, cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(d, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return sfail(COSMOS_ECUDA, std::string("interface evaluation: ") + cudaGetErrorString(e));
    return COSMOS_OK;
}

}  // extern "C"
