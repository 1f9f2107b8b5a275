// Starting guesses for point location in a curvilinear vertex grid.
#pragma once

#include <stdint.h>

namespace rg {

// Approximate cell (ci, cj) of point (px, py) in the grid of nx x ny
// vertices X, Y (row-major): Newton's method on the bilinear index map with
// its analytic Jacobian, in float32 except the corner-minus-point
// differences, which are taken in float64 so that coordinates with a large
// common offset keep their precision.  It is only a starting guess: callers
// confirm it with the exact containment test and walk from it, so its
// rounding never reaches a result.
__device__ __forceinline__ void seed_cell(const double* __restrict__ X, const double* __restrict__ Y, int64_t nx,
                                          int64_t ny, double px, double py, int64_t* ci, int64_t* cj) {
    const int64_t ncx = nx - 1, ncy = ny - 1;
    float fi = 0.5f * (float)ncx, fj = 0.5f * (float)ncy;
    for (int it = 0; it < 16; it++) {
        int64_t i0 = (int64_t)floorf(fi), j0 = (int64_t)floorf(fj);
        i0 = i0 < 0 ? 0 : (i0 > ncx - 1 ? ncx - 1 : i0);
        j0 = j0 < 0 ? 0 : (j0 > ncy - 1 ? ncy - 1 : j0);
        const float dx = fi - (float)i0, dy = fj - (float)j0;
        const int64_t v00 = i0 * ny + j0, v01 = v00 + 1, v10 = v00 + ny, v11 = v10 + 1;
        const float x00 = (float)(__ldg(X + v00) - px), x01 = (float)(__ldg(X + v01) - px);
        const float x10 = (float)(__ldg(X + v10) - px), x11 = (float)(__ldg(X + v11) - px);
        const float y00 = (float)(__ldg(Y + v00) - py), y01 = (float)(__ldg(Y + v01) - py);
        const float y10 = (float)(__ldg(Y + v10) - py), y11 = (float)(__ldg(Y + v11) - py);
        const float ex = (x00 * (1.f - dy) + x01 * dy) * (1.f - dx) + (x10 * (1.f - dy) + x11 * dy) * dx;
        const float ey = (y00 * (1.f - dy) + y01 * dy) * (1.f - dx) + (y10 * (1.f - dy) + y11 * dy) * dx;
        const float xi = (x10 - x00) * (1.f - dy) + (x11 - x01) * dy;
        const float xj = (x01 - x00) * (1.f - dx) + (x11 - x10) * dx;
        const float yi = (y10 - y00) * (1.f - dy) + (y11 - y01) * dy;
        const float yj = (y01 - y00) * (1.f - dx) + (y11 - y10) * dx;
        const float det = xi * yj - xj * yi;
        if (!(det != 0.f) || !isfinite(det)) break;
        const float di = (yj * ex - xj * ey) / det, dj = (-yi * ex + xi * ey) / det;
        if (!isfinite(di) || !isfinite(dj)) break;
        fi = fminf(fmaxf(fi - di, 0.f), (float)ncx);
        fj = fminf(fmaxf(fj - dj, 0.f), (float)ncy);
        if (fabsf(di) < 1e-2f && fabsf(dj) < 1e-2f) break;
    }
    int64_t i = (int64_t)floorf(fi), j = (int64_t)floorf(fj);
    *ci = i < 0 ? 0 : (i >= ncx ? ncx - 1 : i);
    *cj = j < 0 ? 0 : (j >= ncy ? ncy - 1 : j);
}

}  // namespace rg
