/*
 * Small dense solvers standing in for the four LAPACKE routines the reference
 * calls (utils/src/glass_math.c:475-499, 501-571, 590-628).  Row-major only.
 *
 * LAPACKE_dgeev is only reached through matrix_eigenstuff() on the symmetric
 * 8x8 Fisher matrix, so it is implemented as a cyclic Jacobi eigen-solver for
 * symmetric input: wi = 0, and the left and right eigenvectors coincide
 * (stored as columns).  The ordering of the eigenpairs is Jacobi's, not
 * LAPACK's, so eigen-decompositions are compared up to order and sign.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "lapacke.h"

int LAPACKE_dgeev(int layout, char jobvl, char jobvr, int n, double *a, int lda,
                  double *wr, double *wi, double *vl, int ldvl, double *vr, int ldvr)
{
    (void)layout; (void)jobvl; (void)jobvr;
    double *m = malloc(sizeof(double) * n * n);
    double *v = malloc(sizeof(double) * n * n);
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            m[i * n + j] = 0.5 * (a[i * lda + j] + a[j * lda + i]);
            v[i * n + j] = (i == j) ? 1.0 : 0.0;
        }
    for (int sweep = 0; sweep < 100; sweep++) {
        double off = 0.0;
        for (int p = 0; p < n; p++)
            for (int q = p + 1; q < n; q++) off += m[p * n + q] * m[p * n + q];
        if (off == 0.0) break;
        for (int p = 0; p < n; p++) {
            for (int q = p + 1; q < n; q++) {
                double apq = m[p * n + q];
                if (apq == 0.0) continue;
                double theta = (m[q * n + q] - m[p * n + p]) / (2.0 * apq);
                double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; k++) {
                    double mkp = m[k * n + p], mkq = m[k * n + q];
                    m[k * n + p] = c * mkp - s * mkq;
                    m[k * n + q] = s * mkp + c * mkq;
                }
                for (int k = 0; k < n; k++) {
                    double mpk = m[p * n + k], mqk = m[q * n + k];
                    m[p * n + k] = c * mpk - s * mqk;
                    m[q * n + k] = s * mpk + c * mqk;
                }
                for (int k = 0; k < n; k++) {
                    double vkp = v[k * n + p], vkq = v[k * n + q];
                    v[k * n + p] = c * vkp - s * vkq;
                    v[k * n + q] = s * vkp + c * vkq;
                }
            }
        }
    }
    for (int i = 0; i < n; i++) {
        wr[i] = m[i * n + i];
        wi[i] = 0.0;
        for (int j = 0; j < n; j++) {
            if (vl) vl[i * ldvl + j] = v[i * n + j];
            if (vr) vr[i * ldvr + j] = v[i * n + j];
        }
    }
    free(m);
    free(v);
    return 0;
}

/* LAPACK semantics: a zero pivot is recorded in the return value (the first
 * one, 1-based) and the factorisation carries on without scaling that column,
 * so ipiv is always filled. */
int LAPACKE_dgetrf(int layout, int mrows, int n, double *a, int lda, int *ipiv)
{
    (void)layout;
    int info = 0;
    int kmax = mrows < n ? mrows : n;
    for (int k = 0; k < kmax; k++) {
        int piv = k;
        for (int i = k + 1; i < mrows; i++)
            if (fabs(a[i * lda + k]) > fabs(a[piv * lda + k])) piv = i;
        ipiv[k] = piv + 1;
        if (piv != k)
            for (int j = 0; j < n; j++) {
                double t = a[k * lda + j]; a[k * lda + j] = a[piv * lda + j]; a[piv * lda + j] = t;
            }
        if (a[k * lda + k] == 0.0) {
            if (!info) info = k + 1;
            continue;
        }
        for (int i = k + 1; i < mrows; i++) {
            a[i * lda + k] /= a[k * lda + k];
            for (int j = k + 1; j < n; j++) a[i * lda + j] -= a[i * lda + k] * a[k * lda + j];
        }
    }
    return info;
}

/* LAPACK semantics: a singular U (a zero on its diagonal) returns that index
 * and leaves a unchanged. */
int LAPACKE_dgetri(int layout, int n, double *a, int lda, const int *ipiv)
{
    (void)layout;
    for (int i = 0; i < n; i++)
        if (a[i * lda + i] == 0.0) return i + 1;
    double *inv = calloc((size_t)n * n, sizeof(double));
    for (int col = 0; col < n; col++) {
        double *x = inv + (size_t)col * n; /* column stored contiguously */
        for (int i = 0; i < n; i++) x[i] = (i == col) ? 1.0 : 0.0;
        /* apply the row swaps of P to e_col */
        for (int k = 0; k < n; k++) {
            int p = ipiv[k] - 1;
            if (p != k) { double t = x[k]; x[k] = x[p]; x[p] = t; }
        }
        for (int i = 0; i < n; i++)
            for (int j = 0; j < i; j++) x[i] -= a[i * lda + j] * x[j];
        for (int i = n - 1; i >= 0; i--) {
            for (int j = i + 1; j < n; j++) x[i] -= a[i * lda + j] * x[j];
            x[i] /= a[i * lda + i];
        }
    }
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) a[i * lda + j] = inv[(size_t)j * n + i];
    free(inv);
    return 0;
}

int LAPACKE_dpotrf(int layout, char uplo, int n, double *a, int lda)
{
    (void)layout; (void)uplo;
    for (int j = 0; j < n; j++) {
        double d = a[j * lda + j];
        for (int k = 0; k < j; k++) d -= a[j * lda + k] * a[j * lda + k];
        if (d <= 0.0) return j + 1;
        d = sqrt(d);
        a[j * lda + j] = d;
        for (int i = j + 1; i < n; i++) {
            double s = a[i * lda + j];
            for (int k = 0; k < j; k++) s -= a[i * lda + k] * a[j * lda + k];
            a[i * lda + j] = s / d;
        }
    }
    return 0;
}
