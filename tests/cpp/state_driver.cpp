// The state-level classes of include/cosmos_gb300_compat.hpp (state-vector methods, SlopeLimiters, the
// equations of state) from C++: writes their results as raw doubles to argv[1] for
// tests/test_gpu_state.py to compare with the oracle.
#include <cstdio>
#include <vector>

#include "cosmos_gb300_compat.hpp"

int main(int argc, char** argv) {
    if (argc < 2) return 1;
    EulerMaterialParameters mp(1.4);
    EulerStateVector s(0.8, 0.3, -0.2, 0.1, 0.6);
    std::vector<double> out = s.computeConservedVariableVector(mp);
    std::vector<double> f = s.computeXFluxVector(mp);
    out.insert(out.end(), f.begin(), f.end());
    EulerStateVector t;
    t.setConservedVariableVector(s.computeConservedVariableVector(mp), mp);
    std::vector<double> tp = t.computePrimitiveVariableVector();
    out.insert(out.end(), tp.begin(), tp.end());
    out.push_back(SlopeLimiters::computeSlopeLimiter(0.7, 0.0, 1));
    out.push_back(EulerEquationOfState::computeSoundSpeed(0.8, 0.6, mp));
    out.push_back(RelativisticEulerEquationOfState::computeSoundSpeed(1.0, 1.0, EulerMaterialParameters(5.0 / 3.0)));
    FILE* fo = std::fopen(argv[1], "wb");
    if (!fo) return 2;
    std::fwrite(out.data(), sizeof(double), out.size(), fo);
    std::fclose(fo);
    return 0;
}
