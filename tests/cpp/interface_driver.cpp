// Calls the reference-named per-interface solver functions of include/cosmos_gb300_compat.hpp
// (computeXSLICFlux, computeLaxFriedrichsFlux, evolveStateByHalfXTimeStep, the forcing solver's
// evolveConservedVariableVector, ...) one item at a time, as code written against the reference
// does, on the cases of a binary file:
//   per case: int32 op, system, n, width, has_xyz; float64 gamma, dx, dt, bias, frac, bh[5]; int32 lim, side;
//   float64 in[n * width]; float64 xyz[n * 3] if has_xyz
// and writes the 5 outputs of every item, case after case, as float64 to the output file.
// Two more case kinds exercise the black-hole classes: op 100, BlackHoleSpacetime's metric methods
// at points (width 3: x, y, z; dx is the derivative spacing), 125 outputs per item in the layout of
// the COSMOS_ST_* offsets; op 101, BlackHoleEulerEigenvalues of primitives at points (width 8:
// rho, vx, vy, vz, p, x, y, z), 9 outputs per item (material, fast, slow).
//     interface_driver cases.bin out.bin
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <vector>

#include "cosmos_gb300_compat.hpp"

using std::vector;

namespace {

template <class T> T rd(FILE* f) {
    T v;
    if (fread(&v, sizeof v, 1, f) != 1) throw std::runtime_error("truncated case file");
    return v;
}
vector<double> rdv(FILE* f, size_t n) {
    vector<double> v(n);
    if (n && fread(v.data(), sizeof(double), n, f) != n) throw std::runtime_error("truncated case file");
    return v;
}
vector<double> slice(const vector<double>& a, size_t k) { return vector<double>(a.begin() + 5 * k, a.begin() + 5 * k + 5); }
template <class S> S st(const vector<double>& a, size_t k) { return S(a[5 * k], a[5 * k + 1], a[5 * k + 2], a[5 * k + 3], a[5 * k + 4]); }
template <class S> vector<double> prims(S s) { return s.computePrimitiveVariableVector(); }

// Newtonian and SR state forms; V is the item's inputs
template <class S, class Solvers, class First, class Second>
vector<double> flat(int op, const vector<double>& V, double dx, double dt, double bias, int lim, int side,
                    EulerMaterialParameters mp) {
    switch (op) {
        case 6: return First::computeXLaxFriedrichsFlux(st<S>(V, 0), st<S>(V, 1), dx, dt, mp);
        case 7: return First::computeYLaxFriedrichsFlux(st<S>(V, 0), st<S>(V, 1), dx, dt, mp);
        case 8: return First::computeXRichtmyerFlux(st<S>(V, 0), st<S>(V, 1), dx, dt, mp);
        case 9: return First::computeYRichtmyerFlux(st<S>(V, 0), st<S>(V, 1), dx, dt, mp);
        case 10: return First::computeXFORCEFlux(st<S>(V, 0), st<S>(V, 1), dx, dt, mp);
        case 11: return First::computeYFORCEFlux(st<S>(V, 0), st<S>(V, 1), dx, dt, mp);
        case 12: return Second::computeXSLICFlux(st<S>(V, 0), st<S>(V, 1), st<S>(V, 2), st<S>(V, 3), dx, dt, bias, lim, mp);
        case 13: return Second::computeYSLICFlux(st<S>(V, 0), st<S>(V, 1), st<S>(V, 2), st<S>(V, 3), dx, dt, bias, lim, mp);
        case 14: return prims(Solvers::evolveStateByHalfXTimeStep(st<S>(V, 0), st<S>(V, 1), st<S>(V, 2), dx, dt, bias, lim, side, mp));
        case 15: return prims(Solvers::evolveStateByHalfYTimeStep(st<S>(V, 0), st<S>(V, 1), st<S>(V, 2), dx, dt, bias, lim, side, mp));
        case 16: case 17: return prims(Solvers::evolveStateByHalfTimeStep(slice(V, 0), slice(V, 1), slice(V, 2), side, mp));
    }
    throw std::runtime_error("op not defined for this system");
}

vector<double> black_hole(int op, const vector<double>& V, const double* q, double dx, double dt, double bias, int lim,
                          double frac, int side, EulerMaterialParameters mp, BlackHoleSpacetime bh) {
    typedef BlackHoleEulerStateVector S;
    typedef BlackHoleEulerFirstOrderSolver F;
    typedef BlackHoleEulerSolvers U;
    const double x = q[0], y = q[1], z = q[2];
    switch (op) {
        case 6: return F::computeXLaxFriedrichsFlux(st<S>(V, 0), st<S>(V, 1), x, y, z, dx, dt, mp, bh);
        case 7: return F::computeYLaxFriedrichsFlux(st<S>(V, 0), st<S>(V, 1), x, y, z, dx, dt, mp, bh);
        case 8: return F::computeXRichtmyerFlux(st<S>(V, 0), st<S>(V, 1), x, y, z, dx, dt, mp, bh);
        case 9: return F::computeYRichtmyerFlux(st<S>(V, 0), st<S>(V, 1), x, y, z, dx, dt, mp, bh);
        case 10: return F::computeXFORCEFlux(st<S>(V, 0), st<S>(V, 1), x, y, z, dx, dt, mp, bh);
        case 11: return F::computeYFORCEFlux(st<S>(V, 0), st<S>(V, 1), x, y, z, dx, dt, mp, bh);
        case 12: return BlackHoleEulerSecondOrderSolver::computeXSLICFlux(st<S>(V, 0), st<S>(V, 1), st<S>(V, 2), st<S>(V, 3),
                                                                          dx, dt, bias, lim, x, y, z, mp, bh);
        case 13: return BlackHoleEulerSecondOrderSolver::computeYSLICFlux(st<S>(V, 0), st<S>(V, 1), st<S>(V, 2), st<S>(V, 3),
                                                                          dx, dt, bias, lim, x, y, z, mp, bh);
        case 14: return prims(U::evolveStateByHalfXTimeStep(st<S>(V, 0), st<S>(V, 1), st<S>(V, 2), dx, dt, bias, lim, side, x, y, z, mp, bh));
        case 15: return prims(U::evolveStateByHalfYTimeStep(st<S>(V, 0), st<S>(V, 1), st<S>(V, 2), dx, dt, bias, lim, side, x, y, z, mp, bh));
        case 16: return prims(U::evolveStateByHalfXTimeStep(slice(V, 0), slice(V, 1), slice(V, 2), side, dx, x, y, z, mp, bh));
        case 17: return prims(U::evolveStateByHalfYTimeStep(slice(V, 0), slice(V, 1), slice(V, 2), side, dx, x, y, z, mp, bh));
        case 18: return prims(U::evolveStateByFractionalXTimeStep(frac, st<S>(V, 0), st<S>(V, 1), st<S>(V, 2), dx, dt, bias, lim, x, y, z, mp, bh));
        case 19: return prims(U::evolveStateByFractionalYTimeStep(frac, st<S>(V, 0), st<S>(V, 1), st<S>(V, 2), dx, dt, bias, lim, x, y, z, mp, bh));
        case 20: return prims(U::evolveStateByFractionalTimeStep(slice(V, 0), slice(V, 1), x, y, z, mp, bh));
        case 21: return BlackHoleEulerForcingSolver::evolveConservedVariableVector(slice(V, 0), slice(V, 1), slice(V, 2), x, y, z,
                                                                                    dx, dt, bias, lim, mp, bh);
        case 22: return BlackHoleEulerForcingSolver::evolveConservedVariableVector2D(slice(V, 0), slice(V, 1), slice(V, 2),
                                                                                      slice(V, 3), slice(V, 4), x, y, z, dx, dt,
                                                                                      bias, lim, mp, bh);
    }
    throw std::runtime_error("op not defined for the black-hole system");
}

// the vector forms (declared on the Newtonian classes)
vector<double> vectors(int op, const vector<double>& V, double dx, double dt, double frac) {
    switch (op) {
        case 0: return EulerFirstOrderSolver::computeLaxFriedrichsFlux(slice(V, 0), slice(V, 1), slice(V, 2), slice(V, 3), dx, dt);
        case 1: return EulerFirstOrderSolver::computeRichtmyerFlux(slice(V, 0), slice(V, 1), slice(V, 2), slice(V, 3), dx, dt);
        case 2: return EulerFirstOrderSolver::computeFORCEFlux(slice(V, 0), slice(V, 1));
        case 3: return EulerFirstOrderSolver::computeFORCEUpdate(slice(V, 0), slice(V, 1), slice(V, 2), dx, dt);
        case 4: return EulerSolvers::computeFractionalEvolutionVector(frac, slice(V, 0), slice(V, 1), dx, dt);
        case 5: return EulerSolvers::computeEvolutionVector(slice(V, 0), slice(V, 1), dx, dt);
    }
    throw std::runtime_error("not a vector op");
}

vector<double> spacetime(BlackHoleSpacetime bh, double x, double y, double z, double h) {
    vector<double> o;
    auto add = [&](const vector<double>& v) { o.insert(o.end(), v.begin(), v.end()); };
    auto add2 = [&](const vector<vector<double> >& m) { for (auto& r : m) add(r); };
    o.push_back(bh.computeKerrSchildScalar(x, y, z));
    add(bh.computeKerrSchildVector(x, y, z));
    add(bh.computeKerrSchildSpacetimeVector(x, y, z));
    add(bh.computeKerrSchildScalarDerivative(x, y, z, h));
    add2(bh.computeKerrSchildVectorDerivative(x, y, z, h));
    add2(bh.computeSpatialMetricTensor(x, y, z));
    add2(bh.computeSpacetimeMetricTensor(x, y, z));
    add2(bh.computeInverseSpatialMetricTensor(x, y, z));
    add2(bh.computeInverseSpacetimeMetricTensor(x, y, z));
    o.push_back(bh.computeSpatialMetricDeterminant(x, y, z));
    o.push_back(bh.computeSpacetimeMetricDeterminant(x, y, z));
    for (auto& m : bh.computeSpatialMetricTensorDerivative(x, y, z, h)) add2(m);
    o.push_back(bh.computeLapseFunction(x, y, z));
    add(bh.computeShiftVector(x, y, z));
    add(bh.computeLapseFunctionDerivative(x, y, z, h));
    add2(bh.computeShiftVectorDerivative(x, y, z, h));
    add2(bh.computeExtrinsicCurvatureTensor(x, y, z, h));
    o.push_back(bh.inExcisionRegion(x, y, z) ? 1.0 : 0.0);
    return o;
}

vector<double> eigenvalues(const vector<double>& V, EulerMaterialParameters mp, BlackHoleSpacetime bh) {
    vector<double> o;
    auto add = [&](const vector<double>& v) { o.insert(o.end(), v.begin(), v.end()); };
    add(BlackHoleEulerEigenvalues::computeMaterialWaveEigenvalues(V[5], V[6], V[7], V[1], V[2], V[3], mp, bh));
    add(BlackHoleEulerEigenvalues::computeFastAcousticWaveEigenvalues(V[5], V[6], V[7], V[0], V[4], V[1], V[2], V[3], mp, bh));
    add(BlackHoleEulerEigenvalues::computeSlowAcousticWaveEigenvalues(V[5], V[6], V[7], V[0], V[4], V[1], V[2], V[3], mp, bh));
    return o;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 3) {
        fprintf(stderr, "usage: interface_driver cases.bin out.bin\n");
        return 2;
    }
    FILE* f = fopen(argv[1], "rb");
    FILE* o = fopen(argv[2], "wb");
    if (!f || !o) return 2;
    try {
        for (;;) {
            int32_t op;
            if (fread(&op, sizeof op, 1, f) != 1) break;
            const int32_t sys = rd<int32_t>(f), n = rd<int32_t>(f), width = rd<int32_t>(f), has_xyz = rd<int32_t>(f);
            const double gamma = rd<double>(f), dx = rd<double>(f), dt = rd<double>(f), bias = rd<double>(f),
                         frac = rd<double>(f);
            double b[5];
            for (double& v : b) v = rd<double>(f);
            const int32_t lim = rd<int32_t>(f), side = rd<int32_t>(f);
            const vector<double> in = rdv(f, (size_t)n * width);
            const vector<double> xyz = rdv(f, has_xyz ? (size_t)n * 3 : 0);
            EulerMaterialParameters mp(gamma);
            BlackHoleSpacetime bh(b[0], b[1], b[2], b[3], b[4]);
            for (int i = 0; i < n; i++) {
                const vector<double> V(in.begin() + (size_t)i * width, in.begin() + (size_t)(i + 1) * width);
                vector<double> r;
                if (op == 100) r = spacetime(bh, V[0], V[1], V[2], dx);
                else if (op == 101) r = eigenvalues(V, mp, bh);
                else if (op <= 5) r = vectors(op, V, dx, dt, frac);
                else if (sys == 0)
                    r = flat<EulerStateVector, EulerSolvers, EulerFirstOrderSolver, EulerSecondOrderSolver>(op, V, dx, dt, bias, lim, side, mp);
                else if (sys == 1)
                    r = flat<RelativisticEulerStateVector, RelativisticEulerSolvers, RelativisticEulerFirstOrderSolver,
                             RelativisticEulerSecondOrderSolver>(op, V, dx, dt, bias, lim, side, mp);
                else r = black_hole(op, V, &xyz[3 * (size_t)i], dx, dt, bias, lim, frac, side, mp, bh);
                fwrite(r.data(), sizeof(double), r.size(), o);
            }
        }
    } catch (const std::exception& e) {
        fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    fclose(f);
    fclose(o);
    return 0;
}
