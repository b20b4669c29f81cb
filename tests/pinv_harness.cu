// Test harness (host only): runs small_pinv and small_inv of the library's
// scalar header on matrices read from stdin, for tests/test_small_pinv.py.
// Input: count K, then per matrix K*K complex entries (re im, row-major).
// Output per matrix: the rank, then the K*K entries of the pseudo-inverse.
#include <cstdio>

#include "nqes_math.cuh"

int main() {
    int count = 0, K = 0;
    if (std::scanf("%d %d", &count, &K) != 2 || K < 1 || K > 4) return 2;
    for (int c = 0; c < count; c++) {
        nqes::cplx a[16], p[16];
        for (int t = 0; t < K * K; t++)
            if (std::scanf("%lf %lf", &a[t].re, &a[t].im) != 2) return 3;
        const int r = nqes::small_pinv(a, p, K);
        std::printf("%d", r);
        for (int t = 0; t < K * K; t++) std::printf(" %.17g %.17g", p[t].re, p[t].im);
        std::printf("\n");
    }
    return 0;
}
