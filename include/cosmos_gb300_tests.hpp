// The reference's scenario drivers and solution writers (Tests/*.hpp) over the cosmos_gb300 C++
// shim: EulerTests, RelativisticEulerTests, BlackHoleEulerTests, EulerAMRTests and
// RelativisticEulerAMRTests with the reference's method names and arguments.  Each scenario builds
// the reference's initial cells, solves on the GPU (the FP64 path: the reference's numbers) and
// writes density.dat, xVelocity.dat, yVelocity.dat, zVelocity.dat and pressure.dat in the
// reference's text layout.  The reference writes them to a fixed directory of its author's machine;
// here they go to cosmos_tests::output_directory() ("." unless set).
//
// The scenarios are also available as data (cosmos_tests::Problem, from the builders below) so that
// a caller can run them through any solver and write the results with the same writers.
#pragma once

#include <cmath>
#include <fstream>
#include <string>
#include <tuple>
#include <vector>

#include "cosmos_gb300_compat.hpp"

namespace cosmos_tests {

inline std::string& output_directory() {
    static std::string d = ".";
    return d;
}
inline void set_output_directory(const std::string& d) { output_directory() = d; }

// ---------------------------------------------------------------------------------- writers
// Text layout of Tests/EulerTests.cpp:189-252 and its twins: one file per primitive field, numbers
// in the stream's default format (6 significant digits), one line per cell.
struct DatFiles {
    std::ofstream f[5];
    int count;
    explicit DatFiles(int count = 5) : count(count) {
        static const char* names[5] = {"density.dat", "xVelocity.dat", "yVelocity.dat", "zVelocity.dat",
                                       "pressure.dat"};
        for (int k = 0; k < count; k++) f[k].open(output_directory() + "/" + names[k]);
    }
};

template <class S> double field(S s, int k) {
    switch (k) {
        case 0: return s.getDensity();
        case 1: return s.getXVelocity();
        case 2: return s.getYVelocity();
        case 3: return s.getZVelocity();
        default: return s.getPressure();
    }
}

// outputSolution (Tests/EulerTests.cpp:189-214): x = i / n and the value.
template <class S> void write_solution(const std::vector<S>& sol) {
    const long n = (long)sol.size();
    const double dx = 1.0 / n;
    DatFiles d;
    for (int k = 0; k < 5; k++)
        for (long i = 0; i < n; i++) d.f[k] << (dx * i) << " " << field(sol[i], k) << "\n";
}

// outputSolution2D (Tests/EulerTests.cpp:216-252): y = i / rows, x = j / columns, the value; a blank
// line after each row.
template <class S> void write_solution_2d(const std::vector<std::vector<S> >& sol) {
    const long rows = (long)sol.size(), cols = (long)sol[0].size();
    const double rdx = 1.0 / rows, cdx = 1.0 / cols;
    DatFiles d;
    for (int k = 0; k < 5; k++)
        for (long i = 0; i < rows; i++) {
            for (long j = 0; j < cols; j++) d.f[k] << (rdx * i) << " " << (cdx * j) << " " << field(sol[i][j], k) << "\n";
            d.f[k] << "\n";
        }
}

// Black-hole writers (Tests/BlackHoleEulerTests.cpp:201-286): excised cells print 0.
template <class S> void write_solution_bh(const std::vector<S>& sol, const BlackHoleSpacetime& bh) {
    const long n = (long)sol.size();
    const double dx = 1.0 / n;
    DatFiles d;
    for (int k = 0; k < 5; k++)
        for (long i = 0; i < n; i++)
            d.f[k] << (dx * i) << " " << (bh.inExcisionRegion(i * dx, 0.0, 0.0) ? 0.0 : field(sol[i], k)) << "\n";
}
template <class S> void write_solution_bh_2d(const std::vector<std::vector<S> >& sol, const BlackHoleSpacetime& bh) {
    const long rows = (long)sol.size(), cols = (long)sol[0].size();
    const double rdx = 1.0 / rows, cdx = 1.0 / cols;
    DatFiles d;
    for (int k = 0; k < 5; k++)
        for (long i = 0; i < rows; i++) {
            for (long j = 0; j < cols; j++) {
                const double v = bh.inExcisionRegion(j * cdx, i * rdx, 0.0) ? 0.0 : field(sol[i][j], k);
                d.f[k] << (rdx * i) << " " << (cdx * j) << " " << v << "\n";
            }
            d.f[k] << "\n";
        }
}

// Level-1 AMR writer, 1D (Tests/EulerAMRTests.cpp:64-108; the SR twin is the same): an active coarse
// cell, or both fine children at x = (dx / 2)(2i + j) when both are flagged.
template <class S>
void write_level1(const std::vector<S>& c, const std::vector<S>& f, const std::vector<bool>& cf,
                  const std::vector<bool>& ff) {
    const long n = (long)c.size();
    const double dx = 1.0 / n;
    DatFiles d;
    for (int k = 0; k < 5; k++)
        for (long i = 0; i < n; i++) {
            if (cf[i]) {
                d.f[k] << (dx * i) << " " << field(c[i], k) << "\n";
            } else if (ff[i * 2] && ff[i * 2 + 1]) {
                for (int j = 0; j < 2; j++) d.f[k] << ((dx * 0.5) * ((i * 2) + j)) << " " << field(f[i * 2 + j], k) << "\n";
            }
        }
}

// Level-1 AMR writer, 2D (Tests/EulerAMRTests.cpp:208-272): y, x, the cell's two spacings and the
// value, for an active coarse cell or its four flagged children.  The Newtonian class writes all
// five fields; the SR class only the density (Tests/RelativisticEulerAMRTests.cpp:330-370).
template <class S>
void write_level1_2d(const std::vector<std::vector<S> >& c, const std::vector<std::vector<S> >& f,
                     const std::vector<std::vector<bool> >& cf, const std::vector<std::vector<bool> >& ff, int fields) {
    const long rows = (long)c.size(), cols = (long)c[0].size();
    const double rdx = 1.0 / rows, cdx = 1.0 / cols;
    DatFiles d(fields);
    for (int k = 0; k < fields; k++)
        for (long i = 0; i < rows; i++)
            for (long j = 0; j < cols; j++) {
                if (cf[i][j]) {
                    d.f[k] << (rdx * i) << " " << (cdx * j) << " " << rdx << " " << cdx << " " << field(c[i][j], k) << "\n";
                } else if (ff[i * 2][j * 2] && ff[i * 2][j * 2 + 1] && ff[i * 2 + 1][j * 2] && ff[i * 2 + 1][j * 2 + 1]) {
                    for (int a = 0; a < 2; a++)
                        for (int b = 0; b < 2; b++)
                            d.f[k] << ((rdx * 0.5) * ((i * 2) + a)) << " " << ((cdx * 0.5) * ((j * 2) + b)) << " "
                                   << (rdx * 0.5) << " " << (cdx * 0.5) << " " << field(f[i * 2 + a][j * 2 + b], k) << "\n";
                }
            }
}

// Level-2 AMR writer, 1D (Tests/EulerAMRTests.cpp:110-206; the SR twin is the same), following its
// branches: an active coarse cell; else the first intermediate child when flagged, then the second
// or, when that one is not flagged, the two fine cells under it; else the first two fine cells when
// both are flagged, then the last two when both are flagged or else the second intermediate child.
template <class S>
void write_level2(const std::vector<S>& c, const std::vector<S>& m, const std::vector<S>& f, const std::vector<bool>& cf,
                  const std::vector<bool>& mf, const std::vector<bool>& ff) {
    const long n = (long)c.size();
    const double dx = 1.0 / n;
    DatFiles d;
    for (int k = 0; k < 5; k++)
        for (long i = 0; i < n; i++) {
            std::ofstream& o = d.f[k];
            auto fine = [&](long q) { o << ((dx * 0.25) * q) << " " << field(f[q], k) << "\n"; };
            auto mid = [&](long q) { o << ((dx * 0.5) * q) << " " << field(m[q], k) << "\n"; };
            if (cf[i]) {
                o << (dx * i) << " " << field(c[i], k) << "\n";
            } else if (mf[i * 2]) {
                mid(i * 2);
                if (mf[i * 2 + 1]) mid(i * 2 + 1);
                else for (int j = 0; j < 2; j++) fine(i * 4 + 2 + j);
            } else if (ff[i * 4] && ff[i * 4 + 1]) {
                for (int j = 0; j < 2; j++) fine(i * 4 + j);
                if (ff[i * 4 + 2] && ff[i * 4 + 3]) for (int j = 0; j < 2; j++) fine(i * 4 + 2 + j);
                else mid(i * 2 + 1);
            }
        }
}

// Level-2 AMR writer, 2D (Tests/EulerAMRTests.cpp:274-391; the SR twin is the same): density only.
// Written as the reference writes it, including the missing separator between the two spacings of
// the first intermediate cell and the fine spacings printed for the last intermediate cell.
template <class S>
void write_level2_2d(const std::vector<std::vector<S> >& c, const std::vector<std::vector<S> >& m,
                     const std::vector<std::vector<S> >& f, const std::vector<std::vector<bool> >& cf,
                     const std::vector<std::vector<bool> >& mf, const std::vector<std::vector<bool> >& ff) {
    const long rows = (long)c.size(), cols = (long)c[0].size();
    const double rdx = 1.0 / rows, cdx = 1.0 / cols;
    DatFiles d(1);
    std::ofstream& o = d.f[0];
    auto mid = [&](long a, long b) {
        o << ((rdx * 0.5) * a) << " " << ((cdx * 0.5) * b) << " " << (rdx * 0.5) << " " << (cdx * 0.5) << " "
          << field(m[a][b], 0) << "\n";
    };
    auto fine4 = [&](long a0, long b0) {  // the 2 x 2 fine cells from (a0, b0)
        for (int a = 0; a < 2; a++)
            for (int b = 0; b < 2; b++)
                o << ((rdx * 0.25) * (a0 + a)) << " " << ((cdx * 0.25) * (b0 + b)) << " " << (rdx * 0.25) << " "
                  << (cdx * 0.25) << " " << field(f[a0 + a][b0 + b], 0) << "\n";
    };
    auto all4 = [&](long a0, long b0) { return ff[a0][b0] && ff[a0][b0 + 1] && ff[a0 + 1][b0] && ff[a0 + 1][b0 + 1]; };
    for (long i = 0; i < rows; i++)
        for (long j = 0; j < cols; j++) {
            if (cf[i][j]) {
                o << (rdx * i) << " " << (cdx * j) << " " << rdx << " " << cdx << " " << field(c[i][j], 0) << "\n";
            } else if (mf[i * 2][j * 2]) {
                o << ((rdx * 0.5) * (i * 2)) << " " << ((cdx * 0.5) * (j * 2)) << " " << (rdx * 0.5) << (cdx * 0.5) << " "
                  << field(m[i * 2][j * 2], 0) << "\n";
                if (mf[i * 2][j * 2 + 1]) mid(i * 2, j * 2 + 1);
                else fine4(i * 4, j * 4 + 2);
                if (mf[i * 2 + 1][j * 2]) mid(i * 2 + 1, j * 2);
                else fine4(i * 4 + 2, j * 4);
                if (mf[i * 2 + 1][j * 2 + 1]) mid(i * 2 + 1, j * 2 + 1);
                else fine4(i * 4 + 2, j * 4 + 2);
            } else if (all4(i * 4, j * 4)) {
                fine4(i * 4, j * 4);
                if (all4(i * 4 + 2, j * 4 + 2)) {
                    fine4(i * 4 + 2, j * 4 + 2);
                } else {
                    o << ((rdx * 0.5) * ((i * 2) + 1)) << " " << ((cdx * 0.5) * ((j * 2) + 1)) << " " << (rdx * 0.25) << " "
                      << (cdx * 0.25) << " " << field(m[i * 2 + 1][j * 2 + 1], 0) << "\n";
                }
            }
        }
}

// ---------------------------------------------------------------------------------- problems
// One scenario of the reference's Tests/: its initial primitive cells (row-major [ny][nx], 5 per
// cell), spacing 1 / n, material, CFL coefficient, final times and (GR) hole.
struct Problem {
    int system = COSMOS_NEWTONIAN;
    int dims = 1, nx = 0, ny = 1;
    double dx = 0.0, gamma = 1.4, cfl = 0.95;
    double t_final[2] = {0.0, 0.0};  // order 1 (FORCE), order 2 (SLIC)
    double t_amr = 0.0;              // the AMR scenario's final time
    double bh[5] = {1.0, 0.0, 0.5, 0.5, 0.0};
    std::vector<double> prim;
    void set(long c, double r, double u, double v, double w, double p) {
        double* q = &prim[5 * c];
        q[0] = r; q[1] = u; q[2] = v; q[3] = w; q[4] = p;
    }
};

inline Problem make_problem(int system, int dims, int n, double gamma, double t1, double t2, double tamr) {
    Problem P;
    P.system = system;
    P.dims = dims;
    P.nx = n;
    P.ny = dims == 1 ? 1 : n;
    P.dx = 1.0 / n;
    P.gamma = gamma;
    P.t_final[0] = t1;
    P.t_final[1] = t2;
    P.t_amr = tamr;
    P.prim.assign((size_t)5 * P.nx * P.ny, 0.0);
    return P;
}

// distance of cell (i, j) from the grid centre in cells (Tests/EulerTests.cpp:101)
inline double centre_distance(int i, int j, int n) {
    return std::sqrt(((i - (0.5 * n)) * (i - (0.5 * n))) + ((j - (0.5 * n)) * (j - (0.5 * n))));
}

// Toro's tests 1-3, 1D (Tests/EulerTests.cpp:3-88; AMR twins Tests/EulerAMRTests.cpp:3-30).
inline Problem toro_1d(int n, int test) {
    static const double L[3][5] = {{1.0, 0.0, 0.0, 0.0, 1.0}, {1.0, -2.0, 0.0, 0.0, 0.4}, {1.0, 0.0, 0.0, 0.0, 1000.0}};
    static const double R[3][5] = {{0.125, 0.0, 0.0, 0.0, 0.1}, {1.0, 2.0, 0.0, 0.0, 0.4}, {1.0, 0.0, 0.0, 0.0, 0.01}};
    static const double T[3] = {0.25, 0.15, 0.012};
    Problem P = make_problem(COSMOS_NEWTONIAN, 1, n, 1.4, T[test - 1], T[test - 1], T[test - 1]);
    for (int i = 0; i < n; i++) {
        const double* s = i <= (0.5 * n) ? L[test - 1] : R[test - 1];
        P.set(i, s[0], s[1], s[2], s[3], s[4]);
    }
    return P;
}

// Their 2D cylindrical forms (Tests/EulerTests.cpp:90-187; AMR twin Tests/EulerAMRTests.cpp:32-62):
// inside radius 0.2 n the left state, outside the right; test 2 points the velocity radially.
inline Problem toro_2d(int n, int test) {
    static const double T[3] = {0.125, 0.075, 0.006};
    Problem P = make_problem(COSMOS_NEWTONIAN, 2, n, 1.4, T[test - 1], T[test - 1], T[test - 1]);
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            const long c = (long)i * n + j;
            const bool in = centre_distance(i, j, n) <= (0.2 * n);
            if (test == 1) {
                if (in) P.set(c, 1.0, 0.0, 0.0, 0.0, 1.0); else P.set(c, 0.125, 0.0, 0.0, 0.0, 0.1);
            } else if (test == 2) {
                const double th = std::atan2(j - (0.5 * n), i - (0.5 * n));
                if (in) P.set(c, 1.0, -2.0 * std::sin(th), -2.0 * std::cos(th), 0.0, 0.4);
                else P.set(c, 1.0, 2.0 * std::sin(th), 2.0 * std::cos(th), 0.0, 0.4);
            } else {
                if (in) P.set(c, 1.0, 0.0, 0.0, 0.0, 1000.0); else P.set(c, 1.0, 0.0, 0.0, 0.0, 0.01);
            }
        }
    return P;
}

// Special-relativistic tests, 1D (Tests/RelativisticEulerTests.cpp:3-88; AMR twins
// Tests/RelativisticEulerAMRTests.cpp:3-88): 1 mildly relativistic shock, 2 strongly relativistic
// blast, 3 perturbed density.  The shock's SLIC run stops at t = 0.01 where its FORCE run goes to
// 0.4, as in the reference.
inline Problem sr_1d(int n, int test) {
    static const double T[3][3] = {{0.4, 0.01, 0.4}, {0.4, 0.4, 0.4}, {0.35, 0.35, 0.35}};
    Problem P = make_problem(COSMOS_SR, 1, n, 5.0 / 3.0, T[test - 1][0], T[test - 1][1], T[test - 1][2]);
    for (int i = 0; i < n; i++) {
        const bool left = i <= (0.5 * n);
        if (test == 1) {
            if (left) P.set(i, 10.0, 0.0, 0.0, 0.0, 13.3); else P.set(i, 1.0, 0.0, 0.0, 0.0, 0.0);
        } else if (test == 2) {
            if (left) P.set(i, 1.0, 0.0, 0.0, 0.0, 1000.0); else P.set(i, 1.0, 0.0, 0.0, 0.0, 0.01);
        } else {
            if (left) P.set(i, 5.0, 0.0, 0.0, 0.0, 50.0);
            else P.set(i, 2.0 + 0.3 * std::sin(50.0 * (P.dx * i)), 0.0, 0.0, 0.0, 5.0);
        }
    }
    return P;
}

// Their 2D cylindrical forms (Tests/RelativisticEulerTests.cpp:90-187, AMR twins
// Tests/RelativisticEulerAMRTests.cpp:90-187; the AMR blast runs to 0.2 where the plain one stops at
// 0.15).
inline Problem sr_2d(int n, int test) {
    static const double T[3][3] = {{0.2, 0.2, 0.2}, {0.15, 0.15, 0.2}, {0.175, 0.175, 0.175}};
    Problem P = make_problem(COSMOS_SR, 2, n, 5.0 / 3.0, T[test - 1][0], T[test - 1][1], T[test - 1][2]);
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            const long c = (long)i * n + j;
            const bool in = centre_distance(i, j, n) <= (0.2 * n);
            if (test == 1) {
                if (in) P.set(c, 10.0, 0.0, 0.0, 0.0, 13.3); else P.set(c, 1.0, 0.0, 0.0, 0.0, 0.0);
            } else if (test == 2) {
                if (in) P.set(c, 1.0, 0.0, 0.0, 0.0, 1000.0); else P.set(c, 1.0, 0.0, 0.0, 0.0, 0.01);
            } else if (in) {
                P.set(c, 5.0, 0.0, 0.0, 0.0, 50.0);
            } else {
                const double a = P.dx * (i - (0.5 * n)), b = P.dx * (j - (0.5 * n));
                P.set(c, 2.0 + 0.3 * std::sin(50.0 * std::sqrt((a * a) + (b * b))), 0.0, 0.0, 0.0, 5.0);
            }
        }
    return P;
}

// Accretion tests (Tests/BlackHoleEulerTests.cpp:3-197): a dense slab (1D: 0.1 n <= i <= 0.9 n) or
// disc (2D: radius 0.4 n; spheroidal with the axes weighted 0.8 and 1.2) around a Schwarzschild
// (M = 0.05) or spinning (M = 0.1, a = 0.99) hole.  kind: 1 spherical, 2 spinning spherical,
// 3 spheroidal, 4 spinning spheroidal (2D only).
inline Problem bh_problem(int dims, int n, int kind) {
    Problem P = make_problem(COSMOS_GR, dims, n, 5.0 / 3.0, 0.45, 0.45, 0.45);
    const bool spin = kind == 2 || kind == 4;
    const double hole[5] = {spin ? 0.1 : 0.05, spin ? 0.99 : 0.0, 0.5, dims == 1 ? 0.0 : 0.5, 0.0};
    for (int k = 0; k < 5; k++) P.bh[k] = hole[k];
    for (int i = 0; i < P.ny; i++)
        for (int j = 0; j < P.nx; j++) {
            bool dense;
            if (dims == 1) {
                dense = j >= (0.1 * n) && j <= (0.9 * n);
            } else if (kind <= 2) {
                dense = centre_distance(i, j, n) <= 0.4 * n;
            } else {
                dense = std::sqrt(((i - (0.5 * n)) * (i - (0.5 * n)) * 0.8) + ((j - (0.5 * n)) * (j - (0.5 * n)) * 1.2)) <=
                        0.4 * n;
            }
            P.set((long)i * P.nx + j, dense ? 10.0 : 0.1, 0.0, 0.0, 0.0, 0.1);
        }
    return P;
}

// ---------------------------------------------------------------------------------- runs on the GPU
template <class S> std::vector<S> cells_1d(const Problem& P) {
    std::vector<S> v(P.nx);
    cosmos_compat_detail::unpack1(P.prim, v);
    return v;
}
template <class S> std::vector<std::vector<S> > cells_2d(const Problem& P) {
    std::vector<std::vector<S> > g(P.ny, std::vector<S>(P.nx));
    cosmos_compat_detail::unpack2(P.prim, g);
    return g;
}
inline BlackHoleSpacetime hole_of(const Problem& P) { return BlackHoleSpacetime(P.bh[0], P.bh[1], P.bh[2], P.bh[3], P.bh[4]); }

// The plain scenarios: the system's First/SecondOrderSolver::solve(2D) (SLIC with bias 0 and van
// Leer, as every reference scenario calls it), then the writer.
template <class S, class First, class Second>
void run_newtonian_like(const Problem& P, int order) {
    EulerMaterialParameters mp(P.gamma);
    const double T = P.t_final[order == 1 ? 0 : 1];
    if (P.dims == 1) {
        auto c = cells_1d<S>(P);
        write_solution(order == 1 ? First::solve(c, P.dx, P.cfl, T, mp) : Second::solve(c, P.dx, P.cfl, T, 0.0, 1, mp));
    } else {
        auto c = cells_2d<S>(P);
        write_solution_2d(order == 1 ? First::solve2D(c, P.dx, P.cfl, T, mp)
                                     : Second::solve2D(c, P.dx, P.cfl, T, 0.0, 1, mp));
    }
}

inline void run_black_hole(const Problem& P, int order, int sub) {
    EulerMaterialParameters mp(P.gamma);
    const BlackHoleSpacetime h = hole_of(P);
    const double T = P.t_final[order == 1 ? 0 : 1];
    typedef BlackHoleEulerStateVector S;
    if (P.dims == 1) {
        auto c = cells_1d<S>(P);
        write_solution_bh(order == 1 ? BlackHoleEulerFirstOrderSolver::solve(c, P.dx, P.cfl, T, sub, mp, h)
                                     : BlackHoleEulerSecondOrderSolver::solve(c, P.dx, P.cfl, T, 0.0, 1, sub, mp, h), h);
    } else {
        auto c = cells_2d<S>(P);
        write_solution_bh_2d(order == 1 ? BlackHoleEulerFirstOrderSolver::solve2D(c, P.dx, P.cfl, T, sub, mp, h)
                                        : BlackHoleEulerSecondOrderSolver::solve2D(c, P.dx, P.cfl, T, 0.0, 1, sub, mp, h),
                             h);
    }
}

// The AMR scenarios: the system's solveLevel1AMR / solveLevel2AMR (or 2D), then the writer.
template <class S, class Driver>
void run_amr(const Problem& P, int order, double tol, int level, int fields_2d_level1) {
    EulerMaterialParameters mp(P.gamma);
    if (P.dims == 1) {
        auto c = cells_1d<S>(P);
        if (level == 1) {
            auto r = Driver::solveLevel1AMR(c, P.dx, P.cfl, P.t_amr, tol, order, mp);
            write_level1(std::get<0>(r), std::get<1>(r), std::get<2>(r), std::get<3>(r));
        } else {
            auto r = Driver::solveLevel2AMR(c, P.dx, P.cfl, P.t_amr, tol, order, mp);
            write_level2(std::get<0>(r), std::get<1>(r), std::get<2>(r), std::get<3>(r), std::get<4>(r), std::get<5>(r));
        }
    } else {
        auto c = cells_2d<S>(P);
        if (level == 1) {
            auto r = Driver::solve2DLevel1AMR(c, P.dx, P.cfl, P.t_amr, tol, order, mp);
            write_level1_2d(std::get<0>(r), std::get<1>(r), std::get<2>(r), std::get<3>(r), fields_2d_level1);
        } else {
            auto r = Driver::solve2DLevel2AMR(c, P.dx, P.cfl, P.t_amr, tol, order, mp);
            write_level2_2d(std::get<0>(r), std::get<1>(r), std::get<2>(r), std::get<3>(r), std::get<4>(r),
                            std::get<5>(r));
        }
    }
}

}  // namespace cosmos_tests

// ---------------------------------------------------------------------------------- reference names
// Tests/EulerTests.hpp.  solveToroTest4/5 are declared but never defined in the reference; not provided.
class EulerTests {
public:
    static void solveToroTest1(int n, int order) { run(cosmos_tests::toro_1d(n, 1), order); }
    static void solveToroTest2(int n, int order) { run(cosmos_tests::toro_1d(n, 2), order); }
    static void solveToroTest3(int n, int order) { run(cosmos_tests::toro_1d(n, 3), order); }
    static void solve2DToroTest1(int n, int order) { run(cosmos_tests::toro_2d(n, 1), order); }
    static void solve2DToroTest2(int n, int order) { run(cosmos_tests::toro_2d(n, 2), order); }
    static void solve2DToroTest3(int n, int order) { run(cosmos_tests::toro_2d(n, 3), order); }
    static void outputSolution(std::vector<EulerStateVector> s) { cosmos_tests::write_solution(s); }
    static void outputSolution2D(std::vector<std::vector<EulerStateVector> > s) { cosmos_tests::write_solution_2d(s); }
private:
    static void run(const cosmos_tests::Problem& P, int order) {
        cosmos_tests::run_newtonian_like<EulerStateVector, EulerFirstOrderSolver, EulerSecondOrderSolver>(P, order);
    }
};

// Tests/RelativisticEulerTests.hpp
class RelativisticEulerTests {
public:
    static void solveMildlyRelativisticShock(int n, int order) { run(cosmos_tests::sr_1d(n, 1), order); }
    static void solveStronglyRelativisticBlast(int n, int order) { run(cosmos_tests::sr_1d(n, 2), order); }
    static void solvePerturbedDensityTest(int n, int order) { run(cosmos_tests::sr_1d(n, 3), order); }
    static void solve2DMildlyRelativisticShock(int n, int order) { run(cosmos_tests::sr_2d(n, 1), order); }
    static void solve2DStronglyRelativisticBlast(int n, int order) { run(cosmos_tests::sr_2d(n, 2), order); }
    static void solve2DPerturbedDensityTest(int n, int order) { run(cosmos_tests::sr_2d(n, 3), order); }
    static void outputSolution(std::vector<RelativisticEulerStateVector> s) { cosmos_tests::write_solution(s); }
    static void outputSolution2D(std::vector<std::vector<RelativisticEulerStateVector> > s) {
        cosmos_tests::write_solution_2d(s);
    }
private:
    static void run(const cosmos_tests::Problem& P, int order) {
        cosmos_tests::run_newtonian_like<RelativisticEulerStateVector, RelativisticEulerFirstOrderSolver,
                                         RelativisticEulerSecondOrderSolver>(P, order);
    }
};

// Tests/BlackHoleEulerTests.hpp
class BlackHoleEulerTests {
public:
    static void solve1DSphericalAccretionTest(int n, int order, int sub) { run(cosmos_tests::bh_problem(1, n, 1), order, sub); }
    static void solve1DSpinningSphericalAccretionTest(int n, int order, int sub) {
        run(cosmos_tests::bh_problem(1, n, 2), order, sub);
    }
    static void solve2DSphericalAccretionTest(int n, int order, int sub) { run(cosmos_tests::bh_problem(2, n, 1), order, sub); }
    static void solve2DSpinningSphericalAccretionTest(int n, int order, int sub) {
        run(cosmos_tests::bh_problem(2, n, 2), order, sub);
    }
    static void solve2DSpheroidalAccretionTest(int n, int order, int sub) { run(cosmos_tests::bh_problem(2, n, 3), order, sub); }
    static void solve2DSpinningSpheroidalAccretionTest(int n, int order, int sub) {
        run(cosmos_tests::bh_problem(2, n, 4), order, sub);
    }
    static void outputSolution(std::vector<BlackHoleEulerStateVector> s, BlackHoleSpacetime bh) {
        cosmos_tests::write_solution_bh(s, bh);
    }
    static void outputSolution2D(std::vector<std::vector<BlackHoleEulerStateVector> > s, BlackHoleSpacetime bh) {
        cosmos_tests::write_solution_bh_2d(s, bh);
    }
private:
    static void run(const cosmos_tests::Problem& P, int order, int sub) { cosmos_tests::run_black_hole(P, order, sub); }
};

// Tests/EulerAMRTests.hpp (AMRLevel 1 or 2).  Test 2-5 drivers are declared but never defined in the
// reference; not provided.
class EulerAMRTests {
public:
    static void solveToroTest1AMR(int n, int order, double tol, int level) { run(cosmos_tests::toro_1d(n, 1), order, tol, level); }
    static void solve2DToroTest1AMR(int n, int order, double tol, int level) {
        run(cosmos_tests::toro_2d(n, 1), order, tol, level);
    }
private:
    static void run(const cosmos_tests::Problem& P, int order, double tol, int level) {
        cosmos_tests::run_amr<EulerStateVector, EulerAMR>(P, order, tol, level, 5);
    }
};

// Tests/RelativisticEulerAMRTests.hpp (its 2D Level-1 writer writes the density only)
class RelativisticEulerAMRTests {
public:
    static void solveMildlyRelativisticShock(int n, int order, double tol, int level) { run(cosmos_tests::sr_1d(n, 1), order, tol, level); }
    static void solveStronglyRelativisticBlast(int n, int order, double tol, int level) {
        run(cosmos_tests::sr_1d(n, 2), order, tol, level);
    }
    static void solvePerturbedDensityTest(int n, int order, double tol, int level) { run(cosmos_tests::sr_1d(n, 3), order, tol, level); }
    static void solve2DMildlyRelativisticShock(int n, int order, double tol, int level) {
        run(cosmos_tests::sr_2d(n, 1), order, tol, level);
    }
    static void solve2DStronglyRelativisticBlast(int n, int order, double tol, int level) {
        run(cosmos_tests::sr_2d(n, 2), order, tol, level);
    }
    static void solve2DPerturbedDensityTest(int n, int order, double tol, int level) {
        run(cosmos_tests::sr_2d(n, 3), order, tol, level);
    }
private:
    static void run(const cosmos_tests::Problem& P, int order, double tol, int level) {
        cosmos_tests::run_amr<RelativisticEulerStateVector, RelativisticEulerAMR>(P, order, tol, level, 1);
    }
};
