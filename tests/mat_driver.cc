// Test driver for the executable's MAT v5 reader/writer (cli/matv5.cc).
//   mat_driver read <file>   prints every variable: name, dims, complex flag, values
//   mat_driver write <file>  writes a complex 2x3 "a" and a real 2x2x2 "xx"
#include <cstdio>
#include <cstring>
#include <map>
#include <string>

#include "matv5.h"

int main(int argc, char **argv) {
    if (argc != 3) return 2;
    std::string err;
    if (!std::strcmp(argv[1], "read")) {
        std::map<std::string, nqes_cli::MatArray> vars;
        if (!nqes_cli::mat_read(argv[2], vars, err)) {
            std::fprintf(stderr, "%s\n", err.c_str());
            return 1;
        }
        for (auto &[name, a] : vars) {
            std::printf("%s %d %d", name.c_str(), int(a.is_complex), int(a.dims.size()));
            for (auto d : a.dims) std::printf(" %zu", d);
            for (size_t t = 0; t < a.re.size(); t++) {
                std::printf(" %.17g", a.re[t]);
                if (a.is_complex) std::printf(" %.17g", a.im[t]);
            }
            std::printf("\n");
        }
        return 0;
    }
    nqes_cli::MatArray a, xx;
    a.dims = {2, 3};
    a.is_complex = true;
    for (int t = 0; t < 6; t++) {
        a.re.push_back(t + 0.25);
        a.im.push_back(-t - 0.5);
    }
    xx.dims = {2, 2, 2};
    for (int t = 0; t < 8; t++) xx.re.push_back(t * 1.5);
    return nqes_cli::mat_write(argv[2], {{"a", a}, {"xx", xx}}, err) ? 0 : 1;
}
