// Host construction of the block sub-projection matrix (ZQ_InitSubMatPoisson3D,
// Utils3D:1151-1391).  For one s^3 block with faces in the order u (k, j,
// i = 0..s), v (k, j = 0..s, i), w (k = 0..s, j, i):
//   L  the block's Neumann Laplacian (weight 1 between in-block neighbours),
//   P  L without the column of cell 0 (pressure of cell 0 pinned to 0),
//   V  the cell divergence over the block faces,
//   D  the gradient p_b - p_a on interior faces (zero rows on block faces),
// and the matrix is the interior-face rows of I - D [0; P+ V].  P has full
// column rank, so P+ = (P^T P)^-1 P^T; with L symmetric, P^T P is L^2 without
// row and column 0 and P^T V is L V without row 0.  The reference forms P+ with
// an SVD; the normal equations are solved here by Cholesky, in double, and the
// result is rounded to float as the reference stores it.
#include <cmath>
#include <vector>

#include "zqs_coarse.h"

namespace zqs {

std::vector<float> coarse_submatrix(int s) {
    const int n = s * s * s;
    const int nu = s * s * (s + 1);
    const int nf = 3 * nu;
    auto cell = [&](int i, int j, int k) { return (k * s + j) * s + i; };
    auto fu = [&](int i, int j, int k) { return (k * s + j) * (s + 1) + i; };
    auto fv = [&](int i, int j, int k) { return nu + (k * (s + 1) + j) * s + i; };
    auto fw = [&](int i, int j, int k) { return 2 * nu + (k * s + j) * s + i; };

    std::vector<double> L((size_t)n * n, 0.0);
    const int di[6] = {-1, 1, 0, 0, 0, 0}, dj[6] = {0, 0, -1, 1, 0, 0}, dk[6] = {0, 0, 0, 0, -1, 1};
    for (int k = 0; k < s; k++)
        for (int j = 0; j < s; j++)
            for (int i = 0; i < s; i++) {
                const int c = cell(i, j, k);
                int cnt = 0;
                for (int q = 0; q < 6; q++) {
                    const int a = i + di[q], b = j + dj[q], e = k + dk[q];
                    if (a < 0 || a >= s || b < 0 || b >= s || e < 0 || e >= s) continue;
                    L[(size_t)c * n + cell(a, b, e)] = 1.0;
                    cnt++;
                }
                L[(size_t)c * n + c] = -(double)cnt;
            }
    std::vector<double> V((size_t)n * nf, 0.0);
    for (int k = 0; k < s; k++)
        for (int j = 0; j < s; j++)
            for (int i = 0; i < s; i++) {
                double* r = &V[(size_t)cell(i, j, k) * nf];
                r[fu(i, j, k)] -= 1.0;
                r[fu(i + 1, j, k)] += 1.0;
                r[fv(i, j, k)] -= 1.0;
                r[fv(i, j + 1, k)] += 1.0;
                r[fw(i, j, k)] -= 1.0;
                r[fw(i, j, k + 1)] += 1.0;
            }
    const int m = n - 1;
    std::vector<double> G((size_t)m * m, 0.0), B((size_t)m * nf, 0.0);
    for (int a = 1; a < n; a++) {
        for (int b = 1; b < n; b++) {
            double acc = 0.0;
            for (int t = 0; t < n; t++) acc += L[(size_t)a * n + t] * L[(size_t)t * n + b];
            G[(size_t)(a - 1) * m + (b - 1)] = acc;
        }
        for (int t = 0; t < n; t++) {
            const double l = L[(size_t)a * n + t];
            if (l == 0.0) continue;
            const double* vr = &V[(size_t)t * nf];
            double* br = &B[(size_t)(a - 1) * nf];
            for (int q = 0; q < nf; q++) br[q] += l * vr[q];
        }
    }
    // Cholesky G = C C^T (C in the lower triangle of G)
    for (int a = 0; a < m; a++)
        for (int b = 0; b <= a; b++) {
            double acc = G[(size_t)a * m + b];
            for (int t = 0; t < b; t++) acc -= G[(size_t)a * m + t] * G[(size_t)b * m + t];
            if (a == b) G[(size_t)a * m + a] = std::sqrt(acc);
            else G[(size_t)a * m + b] = acc / G[(size_t)b * m + b];
        }
    // X = G^-1 B, column by column (forward then backward substitution)
    for (int q = 0; q < nf; q++) {
        for (int a = 0; a < m; a++) {
            double acc = B[(size_t)a * nf + q];
            for (int t = 0; t < a; t++) acc -= G[(size_t)a * m + t] * B[(size_t)t * nf + q];
            B[(size_t)a * nf + q] = acc / G[(size_t)a * m + a];
        }
        for (int a = m - 1; a >= 0; a--) {
            double acc = B[(size_t)a * nf + q];
            for (int t = a + 1; t < m; t++) acc -= G[(size_t)t * m + a] * B[(size_t)t * nf + q];
            B[(size_t)a * nf + q] = acc / G[(size_t)a * m + a];
        }
    }
    auto pres = [&](int c, int q) -> double { return c == 0 ? 0.0 : B[(size_t)(c - 1) * nf + q]; };
    // interior rows: u (k, j, i = 1..s-1), v (k, j = 1..s-1, i), w (k = 1..s-1, j, i)
    std::vector<float> M;
    M.reserve((size_t)3 * s * s * (s - 1) * nf);
    auto emit = [&](int face, int ca, int cb) {
        for (int q = 0; q < nf; q++) {
            const double v = (q == face ? 1.0 : 0.0) - (pres(cb, q) - pres(ca, q));
            M.push_back((float)v);
        }
    };
    for (int k = 0; k < s; k++)
        for (int j = 0; j < s; j++)
            for (int i = 1; i < s; i++) emit(fu(i, j, k), cell(i - 1, j, k), cell(i, j, k));
    for (int k = 0; k < s; k++)
        for (int j = 1; j < s; j++)
            for (int i = 0; i < s; i++) emit(fv(i, j, k), cell(i, j - 1, k), cell(i, j, k));
    for (int k = 1; k < s; k++)
        for (int j = 0; j < s; j++)
            for (int i = 0; i < s; i++) emit(fw(i, j, k), cell(i, j, k - 1), cell(i, j, k));
    return M;
}

}  // namespace zqs
