// Prints the device stencil of fpm::offset_frame_param (the function the
// illumination update and checkpoint resume use) for (start, offset) cases
// read from stdin: "n m start_row start_col off_row off_col" per line.
// Output per line: valid lower_row lower_col has_upper_row has_upper_col w00 w01 w10 w11.
#include <cstdio>

#include "kernels.h"

int main() {
    int n, m;
    long long sr, sc;
    double orow, ocol;
    while (std::scanf("%d %d %lld %lld %lf %lf", &n, &m, &sr, &sc, &orow, &ocol) == 6) {
        fpm::FrameParam fp{};
        const bool ok = fpm::offset_frame_param(sr, sc, orow, ocol, n, m, fp);
        std::printf("%d %d %d %d %d %.9g %.9g %.9g %.9g\n", ok ? 1 : 0, fp.lower_row, fp.lower_col, fp.has_upper_row,
                    fp.has_upper_col, fp.w00, fp.w01, fp.w10, fp.w11);
    }
    return 0;
}
