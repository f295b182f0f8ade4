/*
 * ddcsvd_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * FP64 CPU restatement of the ddc-svd pipeline (svd_gpu.c:53-131) used as the
 * checker for the CUDA library.  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg load it; the product never does.
 *
 * Stages and the reference code each one follows:
 *   orc_bidiag     Householder Golub-Kahan bidiagonalisation, bidiag.c:33-186
 *                  (same reflector convention: alpha = -sign(x1)||x||,
 *                  H = I - 2 v v^T with ||v|| = 1 stored in place).
 *   orc_dc_sigma   Double divide and conquer singular values,
 *                  Calculations-Parallel.c:706-874 (split K = N/2, merge
 *                  through the secular equation, first/last rows of the
 *                  children's right vectors).  Differences, all deliberate:
 *                  the secular roots are iterated to full FP64 accuracy
 *                  (the reference stops at |g| <= 1e-5, :163,:206); the
 *                  z-hat recomputation uses products of accurately formed
 *                  differences instead of logs (:460-481); sign(z-hat_j) =
 *                  sign(z_j); tiny z_j and equal d_j are deflated (the
 *                  reference has no deflation, :43); the 2x3 leaf uses a
 *                  cancellation-free formula (:626-638); beta[N-1] := 0 (F4).
 *   orc_twisted    Right vectors of B by twisted factorisation,
 *                  parallel-twisted.c:290-528.  The reference factors the
 *                  explicit B^T B - sigma^2 I (which squares the condition
 *                  number); here the factorisations are the stationary and
 *                  progressive differential qd transforms of B^T B = L D L^T
 *                  taken straight from the bidiagonal, which keep relative
 *                  accuracy for small sigma.  Twist index = argmin |gamma|
 *                  (:458-488), vector by the two one-sided recurrences
 *                  (:494-521), then normalisation (:88-123).
 *   orc_left       y = B x / sigma, parallel-twisted.c:530-551 (plus a zero
 *                  guard for sigma = 0, which the reference divides by).
 *   orc_multU/V    Back-transformation, bidiag_par.c:990-1095, with the
 *                  leading-dimension defect of multV for m != n fixed.
 *   orc_svd        The stages in svd_gpu.c:99-121 order.  m < n is handled
 *                  by decomposing A^T.
 *
 * Parity pin: tests/golden holds outputs of the reference's own host code
 * (oracle/_ref) on seeded inputs; the tests check this file against them.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>

#define EPS64 DBL_EPSILON

static int imin(int a, int b) { return a < b ? a : b; }
static double sgn_ref(double x) { return x < 0.0 ? -1.0 : 1.0; } /* bidiag.c:77-82 */

/* ------------------------------------------------------------------------
 * Stage 1: bidiagonalisation (bidiag.c:33-186, both m >= n and m < n).
 * A is column-major with leading dimension lda.
 * ------------------------------------------------------------------------ */
static double col_norm(int len, const double *v) {
    double s = 0.0;
    for (int i = 0; i < len; i++) s += v[i] * v[i];
    return sqrt(s);
}
static double row_norm(int len, const double *v, int ld) {
    double s = 0.0;
    for (int i = 0; i < len; i++) s += v[(size_t)i * ld] * v[(size_t)i * ld];
    return sqrt(s);
}
/* Turns the partial column x (length len, stride inc) into a reflector in
 * place and returns the new diagonal entry (bidiag.c:76-94). */
static double make_reflector(int len, double *x, int inc) {
    double x1 = x[0];
    double s = sgn_ref(x1);
    double nrm = (inc == 1) ? col_norm(len, x) : row_norm(len, x, inc);
    double out = -s * nrm;
    x[0] += s * nrm;
    double scale = sqrt(2.0) * sqrt(nrm * nrm + fabs(nrm * x1));
    double inv = (scale > 0.0) ? 1.0 / scale : 0.0; /* the reference divides by 0 here */
    for (int i = 0; i < len; i++) x[(size_t)i * inc] *= inv;
    return out;
}

/* First `steps` iterations of the main loop only (a bounded timing sample of
 * the same computation; steps >= mn runs the whole reduction). */
int orc_bidiag_steps(int m, int n, double *A, int lda, double *alpha, double *beta, int steps);

int orc_bidiag(int m, int n, double *A, int lda, double *alpha, double *beta) {
    return orc_bidiag_steps(m, n, A, lda, alpha, beta, 1 << 30);
}

int orc_bidiag_steps(int m, int n, double *A, int lda, double *alpha, double *beta, int steps) {
    if (m <= 0 || n <= 0 || lda < m) return 1;
    int mn = imin(m, n);
    for (int i = 0; i < mn - 1; i++) {
        if (i >= steps) return 0;
        double *col = A + i + (size_t)i * lda;
        alpha[i] = make_reflector(m - i, col, 1);
        /* left_householder (bidiag.c:188-218) */
        for (int j = i + 1; j < n; j++) {
            double *c = A + i + (size_t)j * lda;
            double w = 0.0;
            for (int r = 0; r < m - i; r++) w += col[r] * c[r];
            for (int r = 0; r < m - i; r++) c[r] -= 2.0 * col[r] * w;
        }
        double *row = A + i + (size_t)(i + 1) * lda;
        if (i < n - 2) {
            beta[i] = make_reflector(n - i - 1, row, lda);
            /* right_householder (bidiag.c:220-250) */
            for (int r = i + 1; r < m; r++) {
                double *ar = A + r + (size_t)(i + 1) * lda;
                double w = 0.0;
                for (int c = 0; c < n - i - 1; c++) w += row[(size_t)c * lda] * ar[(size_t)c * lda];
                for (int c = 0; c < n - i - 1; c++) ar[(size_t)c * lda] -= 2.0 * row[(size_t)c * lda] * w;
            }
        } else {
            beta[i] = row[0]; /* bidiag.c:125-129 */
            row[0] = 0.0;
        }
    }
    if (n >= m + 1) { /* bidiag.c:133-160 */
        double *row = A + (mn - 1) + (size_t)mn * lda;
        beta[mn - 1] = make_reflector(n - mn, row, lda);
        alpha[mn - 1] = A[(mn - 1) + (size_t)(mn - 1) * lda];
        A[(mn - 1) + (size_t)(mn - 1) * lda] = 0.0;
    } else { /* bidiag.c:161-183 */
        double *col = A + (mn - 1) + (size_t)(mn - 1) * lda;
        alpha[mn - 1] = make_reflector(m - mn + 1, col, 1);
    }
    return 0;
}

/* ------------------------------------------------------------------------
 * Stage 2: double divide and conquer singular values.
 * ------------------------------------------------------------------------ */

/* Secular root i of 1 + sum_j z_j^2 / (d_j^2 - lambda) = 0 over the sorted,
 * non-deflated (d, z) of length q.  Returns the origin index o (the pole the
 * root is closest to) and tau = lambda - d_o^2, so that lambda - d_j^2 can be
 * formed as tau - (d_j - d_o)(d_j + d_o) without cancellation.
 * Root i lies in (d_i^2, d_{i+1}^2), the last one in (d_{q-1}^2,
 * d_{q-1}^2 + ||z||^2) (Calculations-Parallel.c:127-156, 256-260). */
static void secular_eval(int q, const double *d, const double *z, int o, double tau, int split,
                         double *f, double *psi, double *dpsi, double *phi, double *dphi) {
    double ps = 0.0, dps = 0.0, ph = 0.0, dph = 0.0;
    for (int j = 0; j < q; j++) {
        double del = (d[j] - d[o]) * (d[j] + d[o]) - tau; /* d_j^2 - lambda */
        double t = z[j] / del;
        if (j <= split) { ps += z[j] * t; dps += t * t; }
        else { ph += z[j] * t; dph += t * t; }
    }
    *psi = ps; *dpsi = dps; *phi = ph; *dphi = dph;
    *f = 1.0 + ps + ph;
}

static int secular_root(int q, const double *d, const double *z, double zz, int i,
                        int *origin, double *tau_out) {
    const int maxit = 80;
    double f, psi, dpsi, phi, dphi;
    if (i < q - 1) {
        double dd = (d[i + 1] - d[i]) * (d[i + 1] + d[i]);
        /* which pole is closer: sign of f at the midpoint */
        secular_eval(q, d, z, i, 0.5 * dd, i, &f, &psi, &dpsi, &phi, &dphi);
        int o = (f >= 0.0) ? i : i + 1;
        double lo, hi, tau;
        if (o == i) { lo = 0.0; hi = 0.5 * dd; tau = 0.5 * dd; }
        else { lo = -0.5 * dd; hi = 0.0; tau = -0.5 * dd; }
        double da0 = (d[i] - d[o]) * (d[i] + d[o]);
        double db0 = (d[i + 1] - d[o]) * (d[i + 1] + d[o]);
        for (int it = 0; it < maxit; it++) {
            secular_eval(q, d, z, o, tau, i, &f, &psi, &dpsi, &phi, &dphi);
            double err = 8.0 * (1.0 + fabs(psi) + fabs(phi)) + fabs(tau) * (dpsi + dphi);
            if (fabs(f) <= EPS64 * err) break;
            if (f < 0.0) lo = tau; else hi = tau;
            if (hi - lo <= 4.0 * EPS64 * fmax(fabs(lo), fabs(hi))) break;
            /* two-pole rational model through value and slope (middle way) */
            double da = da0 - tau, db = db0 - tau; /* da < 0 < db */
            double s1 = da * da * dpsi, s2 = db * db * dphi;
            double c = f - s1 / da - s2 / db;
            double a_q = c, b_q = c * (da + db) + s1 + s2, c_q = da * db * f;
            double eta;
            double disc = sqrt(fabs(b_q * b_q - 4.0 * a_q * c_q));
            if (a_q == 0.0) eta = c_q / b_q;
            else if (b_q <= 0.0) eta = (b_q - disc) / (2.0 * a_q);
            else eta = 2.0 * c_q / (b_q + disc);
            double tn = tau + eta;
            if (!(tn > lo && tn < hi)) tn = 0.5 * (lo + hi);
            tau = tn;
        }
        *origin = o; *tau_out = tau;
        return 0;
    }
    /* last root: one pole at d_{q-1}, bracket (0, ||z||^2] */
    int o = q - 1;
    double lo = 0.0, hi = zz, tau = 0.5 * zz;
    for (int it = 0; it < maxit; it++) {
        secular_eval(q, d, z, o, tau, q - 1, &f, &psi, &dpsi, &phi, &dphi);
        double err = 8.0 * (1.0 + fabs(psi)) + fabs(tau) * dpsi;
        if (fabs(f) <= EPS64 * err) break;
        if (f < 0.0) lo = tau; else hi = tau;
        if (hi - lo <= 4.0 * EPS64 * fmax(fabs(lo), fabs(hi))) break;
        double da = -tau;
        double s1 = da * da * dpsi;
        double c = f - s1 / da;
        double tn = (c != 0.0) ? tau + da + s1 / c : 0.5 * (lo + hi);
        if (!(tn > lo && tn < hi)) tn = 0.5 * (lo + hi);
        tau = tn;
    }
    *origin = o; *tau_out = tau;
    return 0;
}

typedef struct { double sig; double f; double l; } dc_entry;

/* Merge step of one node.  Inputs (length nn, index 0 = the new d = 0 entry):
 * d (children's singular values, not sorted across the two children), z, and
 * hf/hl = first/last rows of the children's right-vector matrix.  Outputs in
 * ascending sigma order: sig, and (if want_rows) the first/last rows of the
 * merged right vectors.  Calculations-Parallel.c:48-588. */
static int dc_merge(int nn, const double *d_in, const double *z_in, const double *hf_in,
                    const double *hl_in, double *sig_out, double *f_out, double *l_out,
                    int want_rows) {
    int *ord = (int *)malloc(sizeof(int) * nn);
    double *d = (double *)malloc(sizeof(double) * nn);
    double *z = (double *)malloc(sizeof(double) * nn);
    double *hf = (double *)malloc(sizeof(double) * nn);
    double *hl = (double *)malloc(sizeof(double) * nn);
    int *defl = (int *)calloc(nn, sizeof(int));
    /* stable sort by d (insertion into order; entry 0 stays first since d=0) */
    for (int i = 0; i < nn; i++) ord[i] = i;
    for (int i = 1; i < nn; i++) {
        int k = ord[i], j = i - 1;
        while (j >= 0 && d_in[ord[j]] > d_in[k]) { ord[j + 1] = ord[j]; j--; }
        ord[j + 1] = k;
    }
    double dmax = 0.0, zmax = 0.0;
    for (int i = 0; i < nn; i++) {
        d[i] = d_in[ord[i]]; z[i] = z_in[ord[i]]; hf[i] = hf_in[ord[i]]; hl[i] = hl_in[ord[i]];
        dmax = fmax(dmax, fabs(d[i])); zmax = fmax(zmax, fabs(z[i]));
    }
    double tol = 8.0 * EPS64 * fmax(dmax, zmax);
    /* deflation 1: negligible z_j (sigma = d_j, vector = e_j) */
    for (int i = 0; i < nn; i++) if (fabs(z[i]) <= tol) defl[i] = 1;
    /* deflation 2: (nearly) equal d_j -- rotate z_j into its right neighbour */
    int prev = -1;
    for (int i = 0; i < nn; i++) {
        if (defl[i]) continue;
        if (prev >= 0 && d[i] - d[prev] <= tol) {
            double r = hypot(z[prev], z[i]);
            double c = z[i] / r, s = z[prev] / r;
            z[i] = r; z[prev] = 0.0; defl[prev] = 1;
            double f1 = hf[prev], f2 = hf[i], l1 = hl[prev], l2 = hl[i];
            hf[prev] = c * f1 - s * f2; hf[i] = s * f1 + c * f2;
            hl[prev] = c * l1 - s * l2; hl[i] = s * l1 + c * l2;
        }
        prev = i;
    }
    int q = 0;
    for (int i = 0; i < nn; i++) if (!defl[i]) q++;
    double *dq = (double *)malloc(sizeof(double) * (q + 1));
    double *zq = (double *)malloc(sizeof(double) * (q + 1));
    double *fq = (double *)malloc(sizeof(double) * (q + 1));
    double *lq = (double *)malloc(sizeof(double) * (q + 1));
    double *tau = (double *)malloc(sizeof(double) * (q + 1));
    double *zh = (double *)malloc(sizeof(double) * (q + 1));
    int *org = (int *)malloc(sizeof(int) * (q + 1));
    dc_entry *ent = (dc_entry *)malloc(sizeof(dc_entry) * nn);
    int k = 0;
    double zz = 0.0;
    for (int i = 0; i < nn; i++) if (!defl[i]) {
        dq[k] = d[i]; zq[k] = z[i]; fq[k] = hf[i]; lq[k] = hl[i]; zz += z[i] * z[i]; k++;
    }
    /* secular roots (Calculations-Parallel.c:114-344) */
#pragma omp parallel for schedule(dynamic, 8)
    for (int i = 0; i < q; i++) secular_root(q, dq, zq, zz, i, &org[i], &tau[i]);
    int ne = 0;
    if (want_rows && q > 0) {
        /* z-hat by Gu-Eisenstat (Calculations-Parallel.c:460-481, product form) */
#pragma omp parallel for schedule(static)
        for (int j = 0; j < q; j++) {
            int ol = org[q - 1];
            double p = tau[q - 1] - (dq[j] - dq[ol]) * (dq[j] + dq[ol]); /* sigma_{q-1}^2 - d_j^2 */
            for (int kk = 0; kk < j; kk++) {
                int ok = org[kk];
                double num = tau[kk] - (dq[j] - dq[ok]) * (dq[j] + dq[ok]);
                double den = (dq[kk] - dq[j]) * (dq[kk] + dq[j]);
                p *= num / den;
            }
            for (int kk = j; kk < q - 1; kk++) {
                int ok = org[kk];
                double num = tau[kk] - (dq[j] - dq[ok]) * (dq[j] + dq[ok]);
                double den = (dq[kk + 1] - dq[j]) * (dq[kk + 1] + dq[j]);
                p *= num / den;
            }
            double a = sqrt(fabs(p));
            zh[j] = (zq[j] >= 0.0) ? a : -a;
        }
        /* rows of the merged right vectors (Calculations-Parallel.c:489-584) */
#pragma omp parallel for schedule(static)
        for (int i = 0; i < q; i++) {
            int oi = org[i];
            double nv = 0.0, sf = 0.0, sl = 0.0;
            for (int j = 0; j < q; j++) {
                double del = (dq[j] - dq[oi]) * (dq[j] + dq[oi]) - tau[i]; /* d_j^2 - sigma_i^2 */
                double v = zh[j] / del;
                nv += v * v; sf += v * fq[j]; sl += v * lq[j];
            }
            nv = sqrt(nv);
            ent[i].f = sf / nv; ent[i].l = sl / nv;
        }
    }
    for (int i = 0; i < q; i++) ent[i].sig = sqrt(dq[org[i]] * dq[org[i]] + tau[i]);
    if (!want_rows) for (int i = 0; i < q; i++) { ent[i].f = 0.0; ent[i].l = 0.0; }
    ne = q;
    for (int i = 0; i < nn; i++) if (defl[i]) {
        ent[ne].sig = d[i]; ent[ne].f = hf[i]; ent[ne].l = hl[i]; ne++;
    }
    /* merge the two ascending lists (roots, deflated) into the output */
    int a = 0, b = q, o = 0;
    while (a < q || b < nn) {
        int take_a = (b >= nn) || (a < q && ent[a].sig <= ent[b].sig);
        dc_entry e = take_a ? ent[a++] : ent[b++];
        sig_out[o] = e.sig;
        if (f_out) f_out[o] = e.f;
        if (l_out) l_out[o] = e.l;
        o++;
    }
    free(ord); free(d); free(z); free(hf); free(hl); free(defl); free(dq); free(zq);
    free(fq); free(lq); free(tau); free(zh); free(org); free(ent);
    return q;
}

/* Leaves: 1x2 and 2x3 bidiagonals (Calculations-Parallel.c:590-703). */
static void dc_leaf(int nn, const double *b1, const double *b2, double *sig, double *fr,
                    double *lr, double *phi, double *psi) {
    if (nn == 1) {
        double s = hypot(b1[0], b2[0]);
        sig[0] = s;
        if (s > 0.0) { fr[0] = b1[0] / s; lr[0] = b2[0] / s; *phi = b2[0] / s; *psi = -b1[0] / s; }
        else { fr[0] = 1.0; lr[0] = 0.0; *phi = 0.0; *psi = 1.0; }
        return;
    }
    /* B = [b1 b2 0; 0 b3 b4], G = B B^T = [[a, c], [c, e]] */
    double x1 = b1[0], x2 = b2[0], x3 = b1[1], x4 = b2[1];
    double a = x1 * x1 + x2 * x2, e = x3 * x3 + x4 * x4, c = x2 * x3;
    double det = x1 * x1 * x3 * x3 + x1 * x1 * x4 * x4 + x2 * x2 * x4 * x4;
    double hd = 0.5 * (a - e);
    double rad = hypot(hd, c);
    double lmax = 0.5 * (a + e) + rad;
    double lmin = (lmax > 0.0) ? det / lmax : 0.0;
    double lam[2] = { lmin, lmax };
    for (int k = 0; k < 2; k++) {
        sig[k] = sqrt(lam[k]);
        /* left vector u of G for lam[k]: pick the better-conditioned of two forms */
        double u1a = c, u2a = lam[k] - a;
        double u1b = lam[k] - e, u2b = c;
        double na = hypot(u1a, u2a), nb = hypot(u1b, u2b);
        double u1, u2;
        if (na >= nb && na > 0.0) { u1 = u1a / na; u2 = u2a / na; }
        else if (nb > 0.0) { u1 = u1b / nb; u2 = u2b / nb; }
        else { u1 = (k == 0) ? 0.0 : 1.0; u2 = (k == 0) ? 1.0 : 0.0; }
        /* v = B^T u / sigma: first = b1 u1, last = b4 u2 */
        double v1 = x1 * u1, v2 = x2 * u1 + x3 * u2, v3 = x4 * u2;
        double nv = sqrt(v1 * v1 + v2 * v2 + v3 * v3);
        if (nv > 0.0) { fr[k] = v1 / nv; lr[k] = v3 / nv; }
        else { fr[k] = (k == 0) ? 1.0 : 0.0; lr[k] = 0.0; }
    }
    /* null vector = row1 x row2 */
    double n1 = x2 * x4, n2 = -x1 * x4, n3 = x1 * x3;
    double nn3 = sqrt(n1 * n1 + n2 * n2 + n3 * n3);
    if (nn3 > 0.0) { *phi = n1 / nn3; *psi = n3 / nn3; }
    else { *phi = 0.0; *psi = 1.0; }
}

/* Recursive node over b1[0..nn), b2[0..nn) (an nn x (nn+1) bidiagonal).
 * Calculations-Parallel.c:706-850. */
static void dc_node(int nn, const double *b1, const double *b2, double *sig, double *fr,
                    double *lr, double *phi, double *psi, int want_rows) {
    if (nn <= 2) { dc_leaf(nn, b1, b2, sig, fr, lr, phi, psi); return; }
    int K = nn / 2;
    int n2 = nn - K - 1;
    double *s1 = (double *)malloc(sizeof(double) * K), *f1 = (double *)malloc(sizeof(double) * K);
    double *l1 = (double *)malloc(sizeof(double) * K);
    double *s2 = (double *)malloc(sizeof(double) * (n2 > 0 ? n2 : 1));
    double *f2 = (double *)malloc(sizeof(double) * (n2 > 0 ? n2 : 1));
    double *l2 = (double *)malloc(sizeof(double) * (n2 > 0 ? n2 : 1));
    double phi1, psi1, phi2, psi2;
    dc_node(K, b1, b2, s1, f1, l1, &phi1, &psi1, 1);
    dc_node(n2, b1 + K + 1, b2 + K + 1, s2, f2, l2, &phi2, &psi2, 1);
    double bk1 = b1[K], bk2 = b2[K];
    double r0 = hypot(bk1 * psi1, bk2 * phi2);  /* :769-771 */
    double c0 = (r0 > 0.0) ? bk1 * psi1 / r0 : 1.0;
    double s0 = (r0 > 0.0) ? bk2 * phi2 / r0 : 0.0;
    double *d = (double *)malloc(sizeof(double) * nn), *z = (double *)malloc(sizeof(double) * nn);
    double *hf = (double *)malloc(sizeof(double) * nn), *hl = (double *)malloc(sizeof(double) * nn);
    d[0] = 0.0; z[0] = r0; hf[0] = c0 * phi1; hl[0] = s0 * psi2;  /* :774, :789, :797 */
    for (int l = 0; l < K; l++) { d[1 + l] = s1[l]; z[1 + l] = bk1 * l1[l]; hf[1 + l] = f1[l]; hl[1 + l] = 0.0; }
    for (int l = 0; l < n2; l++) { d[K + 1 + l] = s2[l]; z[K + 1 + l] = bk2 * f2[l]; hf[K + 1 + l] = 0.0; hl[K + 1 + l] = l2[l]; }
    dc_merge(nn, d, z, hf, hl, sig, want_rows ? fr : NULL, want_rows ? lr : NULL, want_rows);
    if (want_rows) {
        *phi = -s0 * phi1;  /* :807-808 */
        *psi = c0 * psi2;
        double nf = (*phi) * (*phi), nl = (*psi) * (*psi); /* :812-845 */
        for (int l = 0; l < nn; l++) { nf += fr[l] * fr[l]; nl += lr[l] * lr[l]; }
        nf = sqrt(nf); nl = sqrt(nl);
        if (nf > 0.0) { for (int l = 0; l < nn; l++) fr[l] /= nf; *phi /= nf; }
        if (nl > 0.0) { for (int l = 0; l < nn; l++) lr[l] /= nl; *psi /= nl; }
    }
    free(s1); free(f1); free(l1); free(s2); free(f2); free(l2); free(d); free(z); free(hf); free(hl);
}

/* sigma (ascending) of the N x (N+1) bidiagonal (b1 diagonal, b2 super-
 * diagonal, both length N; b2[N-1] = 0 describes the square N x N case).
 * Calculations-Parallel.c:852-874. */
int orc_dc_sigma(int N, const double *b1, const double *b2, double *sigma) {
    if (N <= 0) return 1;
    double *fr = (double *)malloc(sizeof(double) * N), *lr = (double *)malloc(sizeof(double) * N);
    double phi, psi;
    dc_node(N, b1, b2, sigma, fr, lr, &phi, &psi, 0);
    free(fr); free(lr);
    return 0;
}

/* ------------------------------------------------------------------------
 * Stage 3: right vectors of the N x N upper bidiagonal (a diag, b super,
 * length N-1) by twisted factorisation of L D L^T - sigma^2 I.
 * X is row-per-vector: component j of vector k at X[k*N + j]
 * (parallel-twisted.c:447-448).
 * ------------------------------------------------------------------------ */
static void twisted_one(int N, const double *a, const double *b, double sig, double *x,
                        double *lp, double *um, double *sp) {
    if (N == 1) { x[0] = 1.0; return; }
    double lam = sig * sig;
    double tiny = DBL_MIN / EPS64;
    /* d_i = a_i^2, l_i = b_i / a_i: B^T B = L D L^T */
    /* stationary transform (top-down): L D L^T - lam = L+ D+ L+^T */
    double s = -lam;
    for (int i = 0; i < N - 1; i++) {
        double ai = a[i];
        double di = ai * ai;
        double li = b[i] / ai;
        double dp = di + s;
        if (fabs(dp) < tiny) dp = -tiny;
        double L = di * li / dp;
        lp[i] = L;
        sp[i] = s;
        s = L * li * s - lam;
    }
    sp[N - 1] = s;
    /* progressive transform (bottom-up): L D L^T - lam = U- D- U-^T, with the
     * twist quantity gamma_r = s_r + p_r + lam */
    double p = a[N - 1] * a[N - 1] - lam;
    int r = N - 1;
    double gbest = fabs(sp[N - 1] + p + lam);
    for (int i = N - 2; i >= 0; i--) {
        double ai = a[i];
        double di = ai * ai;
        double li = b[i] / ai;
        double dm = di * li * li + p;
        if (fabs(dm) < tiny) dm = -tiny;
        double t = di / dm;
        um[i] = li * t;
        p = p * t - lam;
        double g = fabs(sp[i] + p + lam);
        if (g < gbest) { gbest = g; r = i; }
    }
    /* solve N_r z = gamma_r e_r with z_r = 1 (parallel-twisted.c:494-521) */
    x[r] = 1.0;
    for (int i = r - 1; i >= 0; i--) x[i] = -lp[i] * x[i + 1];
    for (int i = r; i < N - 1; i++) x[i + 1] = -um[i] * x[i];
    double nrm = 0.0;
    for (int i = 0; i < N; i++) nrm += x[i] * x[i];
    nrm = sqrt(nrm);
    for (int i = 0; i < N; i++) x[i] /= nrm;
}

int orc_twisted(int N, const double *a, const double *b, const double *sigma, double *X) {
    if (N <= 0) return 1;
    /* a zero diagonal entry would make l_i infinite: floor it (rank-deficient B) */
    double bmax = 0.0;
    for (int i = 0; i < N; i++) bmax = fmax(bmax, fabs(a[i]));
    for (int i = 0; i < N - 1; i++) bmax = fmax(bmax, fabs(b[i]));
    double floor_a = (bmax > 0.0 ? bmax : 1.0) * EPS64 * EPS64;
    double *af = (double *)malloc(sizeof(double) * N);
    for (int i = 0; i < N; i++) af[i] = (fabs(a[i]) < floor_a) ? (a[i] < 0 ? -floor_a : floor_a) : a[i];
#pragma omp parallel
    {
        double *lp = (double *)malloc(sizeof(double) * N);
        double *um = (double *)malloc(sizeof(double) * N);
        double *sp = (double *)malloc(sizeof(double) * N);
#pragma omp for schedule(dynamic, 4)
        for (int k = 0; k < N; k++) twisted_one(N, af, b, sigma[k], X + (size_t)k * N, lp, um, sp);
        free(lp); free(um); free(sp);
    }
    free(af);
    return 0;
}

/* Stage 4: y_k = B x_k / sigma_k (parallel-twisted.c:530-551, 58-86). */
int orc_left(int N, const double *a, const double *b, const double *sigma, const double *X, double *Y) {
#pragma omp parallel for schedule(static)
    for (int k = 0; k < N; k++) {
        const double *x = X + (size_t)k * N;
        double *y = Y + (size_t)k * N;
        double nrm = 0.0;
        for (int i = 0; i < N; i++) {
            y[i] = a[i] * x[i] + (i < N - 1 ? b[i] * x[i + 1] : 0.0);
            nrm += y[i] * y[i];
        }
        double den = (sigma[k] > 0.0) ? sigma[k] : sqrt(nrm);
        if (den > 0.0) for (int i = 0; i < N; i++) y[i] /= den;
    }
    return 0;
}

/* Stage 5: back-transformation with the stored reflectors (m >= n).
 * multU (bidiag_par.c:1046-1095): U_k = H_0 ... H_{n-1} [y_k; 0].
 * multV (bidiag_par.c:990-1043): V_k = G_0 ... G_{n-3} x_k, reading the
 * right reflectors from the rows of A (lda) -- the reference passes A^T
 * but indexes it with the wrong leading dimension when m != n. */
int orc_multU(int m, int n, int k, const double *A, int lda, const double *Y, double *U) {
    for (int i = 0; i < n; i++) U[i] = Y[(size_t)k * n + i];
    for (int i = n; i < m; i++) U[i] = 0.0;
    for (int j = n - 1; j >= 0; j--) {
        const double *v = A + j + (size_t)j * lda;
        double w = 0.0;
        for (int r = 0; r < m - j; r++) w += U[j + r] * v[r];
        for (int r = 0; r < m - j; r++) U[j + r] -= 2.0 * v[r] * w;
    }
    return 0;
}

int orc_multV(int m, int n, int k, const double *A, int lda, const double *X, double *V) {
    for (int i = 0; i < n; i++) V[i] = X[(size_t)k * n + i];
    for (int j = n - 3; j >= 0; j--) {
        const double *v = A + j + (size_t)(j + 1) * lda; /* row j from column j+1, stride lda */
        double w = 0.0;
        for (int c = 0; c < n - j - 1; c++) w += v[(size_t)c * lda] * V[j + 1 + c];
        for (int c = 0; c < n - j - 1; c++) V[j + 1 + c] -= 2.0 * v[(size_t)c * lda] * w;
    }
    return 0;
}

/* Splits the N x N bidiagonal at negligible superdiagonal entries
 * (|b_i| <= 4 eps max|B|, eps = the precision the bidiagonal was computed
 * in), zeroing them, and solves each unreduced block on its own: singular
 * values by D&C, right vectors by twisted factorisation, both restricted to
 * the block.  The reference has no splitting; without it equal singular
 * values of decoupled blocks (identity, diagonal, rank-deficient inputs)
 * get identical twisted vectors.  Output: sigma ascending over all blocks,
 * X row-per-vector (N x N), b zeroed at the split points. */
typedef struct { double s; int k; } sig_idx;
static int cmp_sig(const void *a, const void *b) {
    const sig_idx *x = (const sig_idx *)a, *y = (const sig_idx *)b;
    if (x->s < y->s) return -1;
    if (x->s > y->s) return 1;
    return (x->k < y->k) ? -1 : (x->k > y->k);
}

int orc_bdsvd(int N, const double *a, double *b, double eps, double *sigma, double *X) {
    double bmax = 0.0;
    for (int i = 0; i < N; i++) bmax = fmax(bmax, fabs(a[i]));
    for (int i = 0; i < N - 1; i++) bmax = fmax(bmax, fabs(b[i]));
    double tol = 4.0 * eps * bmax;
    for (int i = 0; i < N - 1; i++) if (fabs(b[i]) <= tol) b[i] = 0.0;
    if (N >= 1) b[N - 1] = 0.0;
    double *sl = (double *)malloc(sizeof(double) * N);
    double *Xl = (double *)calloc((size_t)N * N, sizeof(double));
    sig_idx *ord = (sig_idx *)malloc(sizeof(sig_idx) * N);
    int lo = 0;
    while (lo < N) {
        int hi = lo + 1;
        while (hi < N && b[hi - 1] != 0.0) hi++;
        int nb = hi - lo;
        double *bb = (double *)calloc((size_t)nb, sizeof(double));
        double *xb = (double *)malloc(sizeof(double) * (size_t)nb * nb);
        for (int i = 0; i < nb - 1; i++) bb[i] = b[lo + i];
        orc_dc_sigma(nb, a + lo, bb, sl + lo);
        orc_twisted(nb, a + lo, bb, sl + lo, xb);
        for (int k = 0; k < nb; k++)
            for (int i = 0; i < nb; i++) Xl[(size_t)(lo + k) * N + lo + i] = xb[(size_t)k * nb + i];
        free(bb); free(xb);
        lo = hi;
    }
    for (int k = 0; k < N; k++) { ord[k].s = sl[k]; ord[k].k = k; }
    qsort(ord, N, sizeof(sig_idx), cmp_sig);
    for (int r = 0; r < N; r++) {
        sigma[r] = ord[r].s;
        memcpy(X + (size_t)r * N, Xl + (size_t)ord[r].k * N, sizeof(double) * N);
    }
    free(sl); free(Xl); free(ord);
    return 0;
}

/* Full pipeline in svd_gpu.c:99-121 order (m >= n; m < n through A^T).
 * A (m x n, lda) is overwritten as in the reference.  sigma ascending,
 * U (m x mn, ldu), V (n x mn, ldv). Optional stage outputs: alpha (mn),
 * beta (mn), X, Y (mn*mn, row-per-vector). */
int orc_svd(int m, int n, double *A, int lda, double *sigma, double *U, int ldu, double *V,
            int ldv, double *alpha_o, double *beta_o, double *X_o, double *Y_o) {
    if (m <= 0 || n <= 0) return 1;
    if (m < n) {
        double *AT = (double *)malloc(sizeof(double) * (size_t)n * m);
        for (int j = 0; j < n; j++) for (int i = 0; i < m; i++) AT[j + (size_t)i * n] = A[i + (size_t)j * lda];
        int rc = orc_svd(n, m, AT, n, sigma, V, ldv, U, ldu, alpha_o, beta_o, X_o, Y_o);
        free(AT);
        return rc;
    }
    int N = n;
    double *alpha = (double *)malloc(sizeof(double) * N);
    double *beta = (double *)calloc((size_t)N, sizeof(double)); /* beta[N-1] = 0 (F4) */
    double *X = (double *)malloc(sizeof(double) * (size_t)N * N);
    double *Y = (double *)malloc(sizeof(double) * (size_t)N * N);
    orc_bidiag(m, n, A, lda, alpha, beta);
    if (alpha_o) memcpy(alpha_o, alpha, sizeof(double) * N);
    if (beta_o) memcpy(beta_o, beta, sizeof(double) * N);
    orc_bdsvd(N, alpha, beta, EPS64, sigma, X);
    orc_left(N, alpha, beta, sigma, X, Y);
#pragma omp parallel for schedule(static)
    for (int k = 0; k < N; k++) {
        orc_multU(m, n, k, A, lda, Y, U + (size_t)k * ldu);
        orc_multV(m, n, k, A, lda, X, V + (size_t)k * ldv);
    }
    if (X_o) memcpy(X_o, X, sizeof(double) * (size_t)N * N);
    if (Y_o) memcpy(Y_o, Y, sizeof(double) * (size_t)N * N);
    free(alpha); free(beta); free(X); free(Y);
    return 0;
}
