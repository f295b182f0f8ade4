/*
 * ref_driver.c -- TEST INFRASTRUCTURE ONLY (the checker, never the product).
 *
 * Drives the reference's own host C code, compiled unchanged from its sources
 * by oracle/Makefile into oracle/_ref/libddcsvd_ref.so, through the same stage
 * order as svd_gpu() (svd_gpu.c:99-121).  The reference's OpenCL
 * bidiagonalisation (bidiag_par, bidiag_par.c:34) cannot run without an OpenCL
 * device, so its serial twin bidiag_seq (bidiag.c:33) is called instead;
 * bidiag_dr.c:166-172 is the reference's own check that the two agree to 1e-9.
 *
 * One deliberate change against svd_gpu.c:89: beta gets one extra element set
 * to zero, because GetSingularValues_Parallel reads b2[N-1]
 * (Calculations-Parallel.c:744-745,769) while svd_gpu allocates only n-1
 * entries for m >= n.  Without the pad that read is out of bounds.
 *
 * Outputs follow the reference: sigma ascending, U column i at U + i*m,
 * V column i at V + i*n, and A overwritten with the reflectors.  Stage
 * outputs (alpha, beta, X, Y) are returned too so that tests can pin each
 * stage separately.  Stage wall times (seconds) go to t_stage[0..4]:
 * bidiag, singular values, right vectors, left vectors, back-transform.
 */
#include <stdlib.h>
#include <string.h>
#include <time.h>

void bidiag_seq(int m, int n, double *A, double *alpha, double *beta);
void transpose(const int M, const int N, const double *A, double *AT);
void GetSingularValues_Parallel(int N, double b1[], double b2[], double sigma[]);
void CalcRightSingularVectors(int n, int m, double *A, double *B, double *sigma, double *X);
void RighttoLeftSingularVectors(int n, int m, double *A, double *B, double *sigma, double *X, double *Y);
void multU(int m, int n, int vecnum, double *A_mod, double *Y, double *U);
void multV(int m, int n, int vecnum, double *A_mod, double *X, double *V);

static double now_s(void) {
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

/* The reference's serial bidiagonalisation alone (bidiag.c:33-186). */
int ref_bidiag(int m, int n, double *A, double *alpha, double *beta) {
    if (m <= 0 || n <= 0) return 1;
    bidiag_seq(m, n, A, alpha, beta);
    return 0;
}

int ref_svd(int m, int n, double *A, double *sigma, double *U, double *V,
            double *alpha_out, double *beta_out, double *X_out, double *Y_out,
            double *t_stage) {
    if (m <= 0 || n <= 0) return 1;
    int mn = (m >= n) ? n : m;
    int len_beta = (m >= n) ? n - 1 : m;
    double *AT = (double *)malloc(sizeof(double) * (size_t)m * n);
    double *alpha = (double *)calloc((size_t)mn, sizeof(double));
    double *beta = (double *)calloc((size_t)len_beta + 1, sizeof(double)); /* +1: zero pad */
    double *X = (double *)calloc((size_t)mn * (len_beta + 1), sizeof(double));
    double *Y = (double *)calloc((size_t)mn * mn, sizeof(double));
    if (!AT || !alpha || !beta || !X || !Y) {
        free(AT); free(alpha); free(beta); free(X); free(Y);
        return 2;
    }
    double t0 = now_s();
    bidiag_seq(m, n, A, alpha, beta);
    double t1 = now_s();
    transpose(m, n, A, AT);
    GetSingularValues_Parallel(mn, alpha, beta, sigma);
    double t2 = now_s();
    CalcRightSingularVectors(mn, len_beta + 1, alpha, beta, sigma, X);
    double t3 = now_s();
    RighttoLeftSingularVectors(mn, len_beta + 1, alpha, beta, sigma, X, Y);
    double t4 = now_s();
#pragma omp parallel for default(shared)
    for (int i = 0; i < mn; i++) {
        multU(m, n, i, A, Y, U + (size_t)i * m);
        multV(m, n, i, AT, X, V + (size_t)i * n);
    }
    double t5 = now_s();
    if (t_stage) {
        t_stage[0] = t1 - t0; t_stage[1] = t2 - t1; t_stage[2] = t3 - t2;
        t_stage[3] = t4 - t3; t_stage[4] = t5 - t4;
    }
    if (alpha_out) memcpy(alpha_out, alpha, sizeof(double) * mn);
    if (beta_out) memcpy(beta_out, beta, sizeof(double) * len_beta);
    if (X_out) memcpy(X_out, X, sizeof(double) * (size_t)mn * (len_beta + 1));
    if (Y_out) memcpy(Y_out, Y, sizeof(double) * (size_t)mn * mn);
    free(AT); free(alpha); free(beta); free(X); free(Y);
    return 0;
}
