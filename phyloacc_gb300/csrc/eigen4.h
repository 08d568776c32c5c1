// eigen4.h — real eigendecomposition of a small (n <= 5) substitution-rate
// matrix, header-only, host-side FP64.
//
// PhyloAcc-ST decomposes the RATE_MAT of the .mod file once with Armadillo's
// eig_gen and keeps eigenvec = V^T, eigeninv = (V^T)^-1 and the real parts of
// the eigenvalues (src/PhyloAcc-ST/bpp.hpp:357-362).  Every transition matrix
// of the sampler is then  P^T(t) = eigeninv * diag(exp(lambda*t)) * eigenvec
// (bpp.hpp:375-380, bpp_c.cpp:195-219).  This header computes the same
// eigensystem with project-written numerics:
//   * eigenvalues: Householder reduction to Hessenberg form followed by the
//     shifted QR algorithm with Wilkinson shifts and deflation (Francis 1961;
//     Golub & Van Loan, "Matrix Computations", 4th ed., sections 7.4-7.5);
//   * eigenvectors: a basis of null(Q - lambda I) by Gaussian elimination
//     with complete pivoting, with the rank fixed by the multiplicity of the
//     eigenvalue cluster (handles the repeated spectra of JC69/F81 models);
//   * V^-1: Gauss-Jordan elimination with partial pivoting.
// A complex spectrum (possible only for non-reversible Q) is reported as an
// error instead of silently taking real parts.
#pragma once
#include <cmath>
#include <cstring>
#include <algorithm>

namespace pacc_eigen {

enum { EIG_OK = 0, EIG_COMPLEX = 1, EIG_NOCONV = 2, EIG_SINGULAR = 3, EIG_BADN = 4 };

static const int NMAX = 5;

// Eigenvalues of the 2x2 block [a b; c d]. Returns false if complex.
inline bool eig2x2(double a, double b, double c, double d, double* l1, double* l2) {
    double tr = 0.5 * (a + d);
    double df = 0.5 * (a - d);
    double disc = df * df + b * c;
    double scale = std::fabs(a) + std::fabs(b) + std::fabs(c) + std::fabs(d);
    if (disc < 0) {
        if (-disc > 1e-24 * scale * scale) return false;
        disc = 0;
    }
    double s = std::sqrt(disc);
    *l1 = tr + s;
    *l2 = tr - s;
    return true;
}

// Eigenvalues of the n x n matrix A (row-major).  Returns EIG_OK and fills lam.
inline int eigenvalues(int n, const double* A, double* lam) {
    if (n < 1 || n > NMAX) return EIG_BADN;
    double H[NMAX][NMAX];
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) H[i][j] = A[i * n + j];
    // Householder reduction to upper Hessenberg form.
    for (int k = 0; k < n - 2; k++) {
        double alpha = 0;
        for (int i = k + 1; i < n; i++) alpha += H[i][k] * H[i][k];
        alpha = std::sqrt(alpha);
        if (alpha == 0) continue;
        if (H[k + 1][k] > 0) alpha = -alpha;
        double v[NMAX] = {0};
        v[k + 1] = H[k + 1][k] - alpha;
        for (int i = k + 2; i < n; i++) v[i] = H[i][k];
        double vnorm2 = 0;
        for (int i = k + 1; i < n; i++) vnorm2 += v[i] * v[i];
        if (vnorm2 == 0) continue;
        // H = (I - 2vv^T/|v|^2) H (I - 2vv^T/|v|^2)
        for (int j = 0; j < n; j++) {
            double s = 0;
            for (int i = k + 1; i < n; i++) s += v[i] * H[i][j];
            s = 2 * s / vnorm2;
            for (int i = k + 1; i < n; i++) H[i][j] -= s * v[i];
        }
        for (int i = 0; i < n; i++) {
            double s = 0;
            for (int j = k + 1; j < n; j++) s += H[i][j] * v[j];
            s = 2 * s / vnorm2;
            for (int j = k + 1; j < n; j++) H[i][j] -= s * v[j];
        }
        for (int i = k + 2; i < n; i++) H[i][k] = 0;
    }
    const double eps = 2.220446049250313e-16;
    int hi = n - 1;
    int iter = 0, total = 0;
    while (hi >= 0) {
        if (hi == 0) { lam[0] = H[0][0]; break; }
        int l = hi;
        while (l > 0) {
            double s = std::fabs(H[l][l]) + std::fabs(H[l - 1][l - 1]);
            if (s == 0) s = 1;
            if (std::fabs(H[l][l - 1]) <= eps * s) break;
            l--;
        }
        if (l > 0) H[l][l - 1] = 0;
        if (l == hi) { lam[hi] = H[hi][hi]; hi--; iter = 0; continue; }
        if (l == hi - 1) {
            double l1, l2;
            if (!eig2x2(H[hi - 1][hi - 1], H[hi - 1][hi], H[hi][hi - 1], H[hi][hi], &l1, &l2))
                return EIG_COMPLEX;
            lam[hi - 1] = l1;
            lam[hi] = l2;
            hi -= 2;
            iter = 0;
            continue;
        }
        if (++total > 400) return EIG_NOCONV;
        // Wilkinson shift from the trailing 2x2 of the active block.
        double mu;
        double l1, l2;
        if (eig2x2(H[hi - 1][hi - 1], H[hi - 1][hi], H[hi][hi - 1], H[hi][hi], &l1, &l2))
            mu = (std::fabs(l1 - H[hi][hi]) < std::fabs(l2 - H[hi][hi])) ? l1 : l2;
        else
            mu = H[hi][hi];
        if (iter > 0 && iter % 10 == 0) mu = H[hi][hi] + std::fabs(H[hi][hi - 1]);
        iter++;
        // Explicit shifted QR step on rows/cols l..hi via Givens rotations.
        double cs[NMAX], sn[NMAX];
        for (int i = l; i <= hi; i++) H[i][i] -= mu;
        for (int k = l; k < hi; k++) {
            double a = H[k][k], b = H[k + 1][k];
            double r = std::hypot(a, b);
            double c = (r == 0) ? 1.0 : a / r, s = (r == 0) ? 0.0 : b / r;
            cs[k] = c; sn[k] = s;
            for (int j = k; j <= hi; j++) {
                double t1 = H[k][j], t2 = H[k + 1][j];
                H[k][j] = c * t1 + s * t2;
                H[k + 1][j] = -s * t1 + c * t2;
            }
        }
        for (int k = l; k < hi; k++) {
            double c = cs[k], s = sn[k];
            int top = std::min(k + 2, hi);
            for (int i = l; i <= top; i++) {
                double t1 = H[i][k], t2 = H[i][k + 1];
                H[i][k] = c * t1 + s * t2;
                H[i][k + 1] = -s * t1 + c * t2;
            }
        }
        for (int i = l; i <= hi; i++) H[i][i] += mu;
    }
    return EIG_OK;
}

// Basis of the null space of A (n x n row-major) with the rank fixed to
// n - m.  Writes m vectors as columns of V starting at column col0.
inline void null_basis(int n, const double* A, int m, double* V, int col0) {
    double M[NMAX][NMAX];
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) M[i][j] = A[i * n + j];
    int colperm[NMAX];
    for (int j = 0; j < n; j++) colperm[j] = j;
    int r = n - m;
    for (int k = 0; k < r; k++) {
        int pi = k, pj = k;
        double best = -1;
        for (int i = k; i < n; i++)
            for (int j = k; j < n; j++)
                if (std::fabs(M[i][j]) > best) { best = std::fabs(M[i][j]); pi = i; pj = j; }
        if (pi != k)
            for (int j = 0; j < n; j++) std::swap(M[k][j], M[pi][j]);
        if (pj != k) {
            for (int i = 0; i < n; i++) std::swap(M[i][k], M[i][pj]);
            std::swap(colperm[k], colperm[pj]);
        }
        double piv = M[k][k];
        if (piv == 0) continue;
        for (int i = k + 1; i < n; i++) {
            double f = M[i][k] / piv;
            if (f == 0) continue;
            for (int j = k; j < n; j++) M[i][j] -= f * M[k][j];
        }
    }
    for (int f = 0; f < m; f++) {
        double x[NMAX] = {0};
        x[r + f] = 1.0;
        for (int k = r - 1; k >= 0; k--) {
            double s = 0;
            for (int j = k + 1; j < n; j++) s += M[k][j] * x[j];
            x[k] = (M[k][k] == 0) ? 0.0 : -s / M[k][k];
        }
        double nrm = 0;
        for (int j = 0; j < n; j++) nrm += x[j] * x[j];
        nrm = std::sqrt(nrm);
        for (int j = 0; j < n; j++) V[colperm[j] * n + col0 + f] = x[j] / nrm;
    }
}

// Inverse of the n x n matrix A by Gauss-Jordan with partial pivoting.
inline int invert(int n, const double* A, double* Ainv) {
    double M[NMAX][2 * NMAX];
    for (int i = 0; i < n; i++) {
        for (int j = 0; j < n; j++) { M[i][j] = A[i * n + j]; M[i][n + j] = (i == j) ? 1.0 : 0.0; }
    }
    for (int k = 0; k < n; k++) {
        int p = k;
        for (int i = k + 1; i < n; i++)
            if (std::fabs(M[i][k]) > std::fabs(M[p][k])) p = i;
        if (M[p][k] == 0) return EIG_SINGULAR;
        if (p != k)
            for (int j = 0; j < 2 * n; j++) std::swap(M[k][j], M[p][j]);
        double piv = M[k][k];
        for (int j = 0; j < 2 * n; j++) M[k][j] /= piv;
        for (int i = 0; i < n; i++) {
            if (i == k) continue;
            double f = M[i][k];
            if (f == 0) continue;
            for (int j = 0; j < 2 * n; j++) M[i][j] -= f * M[k][j];
        }
    }
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) Ainv[i * n + j] = M[i][n + j];
    return EIG_OK;
}

// Full decomposition Q = V diag(lam) V^-1.  lam sorted descending.
// V, Vinv: n x n row-major, columns of V are right eigenvectors.
inline int decompose(int n, const double* Q, double* lam, double* V, double* Vinv) {
    int st = eigenvalues(n, Q, lam);
    if (st != EIG_OK) return st;
    std::sort(lam, lam + n, [](double a, double b) { return a > b; });
    double qs = 0;
    for (int i = 0; i < n * n; i++) qs = std::max(qs, std::fabs(Q[i]));
    if (qs == 0) qs = 1;
    int i = 0;
    while (i < n) {
        int j = i + 1;
        while (j < n && std::fabs(lam[j] - lam[i]) <= 1e-9 * qs) j++;
        int m = j - i;
        double mean = 0;
        for (int k = i; k < j; k++) mean += lam[k];
        mean /= m;
        for (int k = i; k < j; k++) lam[k] = (m > 1) ? mean : lam[k];
        double A[NMAX * NMAX];
        for (int r = 0; r < n; r++)
            for (int c = 0; c < n; c++) A[r * n + c] = Q[r * n + c] - ((r == c) ? lam[i] : 0.0);
        null_basis(n, A, m, V, i);
        i = j;
    }
    return invert(n, V, Vinv);
}

}  // namespace pacc_eigen
