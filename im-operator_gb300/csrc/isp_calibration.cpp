// isp_calibration.cpp - colour-correction matrix from patch measurements (host code).
//
// The least-squares solve of the reference's colour calibration (color_calibration::
// process_solve_ccm, src/color_calibration/solve_ccm.cpp:15-119), with the same results: per
// output channel the normal equations (X^T X + 1e-9 I) c = X^T y over the patches, in FP64, solved
// by Gaussian elimination with partial pivoting (src/color_calibration/common.hpp:27-58).  The
// features are (r, g, b) for 3x3, (r, g, b, 1) for 3x4 with bias, and (r, g, b, rg, rb, gb, r^2,
// g^2, b^2) for the 3x9 polynomial.  Its output seeds the CCM of the differentiable chain, whose
// adjoint then fits the matrix on raw frames (imop_gb300.calibration).

#include <cmath>
#include <cstring>
#include <utility>

#include "../../include/imop_isp.h"

namespace {

// A x = b in place (A n x n row-major, b -> x); false when a pivot vanishes
bool gauss_solve(int n, double* A, double* b) {
    for (int col = 0; col < n; col++) {
        int piv = col;
        double best = std::fabs(A[col * n + col]);
        for (int r = col + 1; r < n; r++) {
            const double v = std::fabs(A[r * n + col]);
            if (v > best) best = v, piv = r;
        }
        if (best < 1e-30) return false;
        if (piv != col) {
            for (int j = col; j < n; j++) std::swap(A[col * n + j], A[piv * n + j]);
            std::swap(b[col], b[piv]);
        }
        const double p = A[col * n + col];
        for (int r = col + 1; r < n; r++) {
            const double f = A[r * n + col] / p;
            A[r * n + col] = 0.0;
            for (int j = col + 1; j < n; j++) A[r * n + j] -= f * A[col * n + j];
            b[r] -= f * b[col];
        }
    }
    for (int i = n - 1; i >= 0; i--) {
        double s = b[i];
        for (int j = i + 1; j < n; j++) s -= A[i * n + j] * b[j];
        if (std::fabs(A[i * n + i]) < 1e-30) return false;
        b[i] = s / A[i * n + i];
    }
    return true;
}

int features(const ImopPatchColor& c, int type, double* f) {
    if (type == IMOP_CCM_POLY_3X9) {
        // products of the float channels, widened afterwards (as the reference's initialiser)
        const float r = c.r, g = c.g, b = c.b;
        f[0] = r, f[1] = g, f[2] = b;
        f[3] = r * g, f[4] = r * b, f[5] = g * b;
        f[6] = r * r, f[7] = g * g, f[8] = b * b;
        return 9;
    }
    f[0] = c.r, f[1] = c.g, f[2] = c.b, f[3] = 1.0;
    return type == IMOP_CCM_LINEAR_4X3 ? 4 : 3;
}

}  // namespace

extern "C" int imop_solve_ccm(const ImopPatchColor* measured, const ImopPatchColor* reference, int n, int type,
                              ImopSolvedMatrix* out) {
    if (!measured || !reference || !out) return IMOP_ERR_NULL_INPUT;
    if (n < 3) return IMOP_ERR_INSUFFICIENT_PATCHES;
    if (type != IMOP_CCM_LINEAR_3X3 && type != IMOP_CCM_LINEAR_4X3 && type != IMOP_CCM_POLY_3X9)
        return IMOP_ERR_INVALID_ARGUMENT;
    std::memset(out, 0, sizeof(*out));
    const int K = type == IMOP_CCM_POLY_3X9 ? 9 : (type == IMOP_CCM_LINEAR_4X3 ? 4 : 3);
    out->type = type;
    out->rows = 3;
    out->cols = K;
    for (int ch = 0; ch < 3; ch++) {
        double A[81] = {0}, y[9] = {0}, f[9];
        for (int i = 0; i < n; i++) {
            features(measured[i], type, f);
            const double t = ch == 0 ? reference[i].r : (ch == 1 ? reference[i].g : reference[i].b);
            for (int a = 0; a < K; a++) {
                y[a] += f[a] * t;
                for (int c = 0; c < K; c++) A[a * K + c] += f[a] * f[c];
            }
        }
        for (int a = 0; a < K; a++) A[a * K + a] += 1e-9;
        if (!gauss_solve(K, A, y)) return IMOP_ERR_SINGULAR;
        for (int k = 0; k < K; k++) out->m[ch * K + k] = (float)y[k];
    }
    return IMOP_OK;
}
