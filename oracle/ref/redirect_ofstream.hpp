// Test infrastructure only: compiled ahead of the reference's Tests/*.cpp (by oracle/ref/Makefile)
// so that their output files, which the reference opens at a fixed absolute path of its author's
// machine, land in a directory the harness chooses (ref_tests_set_dir).  Every standard header the
// reference uses is included first; the macro below then renames only the reference's own
// unqualified `ofstream` declarations.  Nothing in the reference's sources is changed.
#include <cmath>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <tuple>
#include <vector>

namespace cosmos_ref_redirect {
// maps an absolute path of the reference to <chosen directory>/<file name>
std::string map_path(const char* path);
}

struct CosmosRedirectOfstream : std::ofstream {
    explicit CosmosRedirectOfstream(const char* path) : std::ofstream(cosmos_ref_redirect::map_path(path)) {}
};
#define ofstream CosmosRedirectOfstream
