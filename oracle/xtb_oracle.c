/*
 * CPU oracle for the GFN2-xTB single point: pair loops in plain C.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is a CPU restatement of the
 * reference algorithm (tblite 0.7.0, Fortran) used to check the CUDA
 * engine.  Only tests/, __graft_entry__.smoke() and the cpu_baseline /
 * reference arms of bench.py may load it.  The product never calls it.
 *
 * Each routine cites the reference routine it restates.  Layout
 * conventions (row-major C):
 *   xyz[nat][3]                       Bohr
 *   S[n][n], H[n][n]                  symmetric AO matrices
 *   D[3][n][n], Q[6][n][n]            D[k][row][col] = <row|(r - R_A(col))_k|col>,
 *                                     i.e. the multipole operator sits on the atom
 *                                     of the column index (the reference stores
 *                                     dpint(k, j, i) with the operator on atom of i).
 *   Q components ordered xx, xy, yy, xz, yz, zz and made traceless
 *   (Q' = 3/2 M - 1/2 tr(M) delta), as the reference does.
 *   spherical p order (y, z, x); spherical d order (xy, yz, z2, xz, x2-y2).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define MAXL 2
#define MAXG 12

static const int NCART[3] = {1, 3, 6};
static const int NSPH[3] = {1, 3, 5};
static const int CEXP[3][6][3] = {
    {{0, 0, 0}},
    {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}},
    {{2, 0, 0}, {1, 1, 0}, {1, 0, 1}, {0, 2, 0}, {0, 1, 1}, {0, 0, 2}}};

/* cartesian -> spherical, reference src/tblite/integral/trafo.f90:36-45,104-253 */
static double TRAFO[3][5][6];
static int trafo_ready = 0;
static void init_trafo(void) {
    if (trafo_ready) return;
    memset(TRAFO, 0, sizeof(TRAFO));
    TRAFO[0][0][0] = 1.0;
    /* p: spherical (y, z, x) */
    TRAFO[1][0][1] = 1.0;
    TRAFO[1][1][2] = 1.0;
    TRAFO[1][2][0] = 1.0;
    const double s3 = sqrt(3.0), s3_4 = 0.5 * sqrt(3.0);
    /* d rows m=-2..2, cartesian xx xy xz yy yz zz */
    TRAFO[2][0][1] = s3;
    TRAFO[2][1][4] = s3;
    TRAFO[2][2][0] = -0.5; TRAFO[2][2][3] = -0.5; TRAFO[2][2][5] = 1.0;
    TRAFO[2][3][2] = s3;
    TRAFO[2][4][0] = s3_4; TRAFO[2][4][3] = -s3_4;
    trafo_ready = 1;
}

static double dfact(int k) { /* (2k-1)!! */
    static const double t[8] = {1, 1, 3, 15, 105, 945, 10395, 135135};
    return t[k];
}

/* Gaussian 1-d moment about the product centre, reference integrals.f90:91-101 */
static double s1d(int m, double eta) {
    if (m & 1) return 0.0;
    return pow(0.5 / eta, m / 2) * dfact(m / 2);
}

static double binom(int n, int k) {
    static const double t[6][6] = {{1}, {1, 1}, {1, 2, 1}, {1, 3, 3, 1}, {1, 4, 6, 4, 1},
                                   {1, 5, 10, 10, 5, 1}};
    return t[n][k];
}

/* 1-d factor of <x_j^b | (x-O)^e | x_i^a> for one primitive pair:
 * (x-A)^a (x-B)^b expanded about P, moment of (x-O)^e, O given by po = P-O. */
static double mom1d(int a, int b, double pa, double pb, double po, int e, double eta) {
    if (a < 0) return 0.0;
    double va[8] = {0}, vb[8] = {0}, vv[16] = {0};
    for (int m = 0; m <= a; ++m) va[m] = binom(a, m) * pow(pa, a - m);
    for (int m = 0; m <= b; ++m) vb[m] = binom(b, m) * pow(pb, b - m);
    for (int i = 0; i <= a; ++i)
        for (int j = 0; j <= b; ++j) vv[i + j] += va[i] * vb[j];
    double res = 0.0;
    for (int m = 0; m <= a + b; ++m) {
        if (vv[m] == 0.0) continue;
        double acc = 0.0;
        for (int t = 0; t <= e; ++t) acc += binom(e, t) * pow(po, e - t) * s1d(m + t, eta);
        res += vv[m] * acc;
    }
    return res;
}

typedef struct {
    int l, nprim;
    double alpha[MAXG], coeff[MAXG];
} cgto_t;

/* Moment integrals of one shell pair: j (bra, on B) and i (ket, on A),
 * vec = R_A - R_B.  Outputs in spherical functions, [mj][mi]:
 *   s, dA[3], qA[6] (operator on A),  dB[3], qB[6] (operator on B).
 * With grad != 0 also d/dR_A (component c) of each:  gs[3], gdA[3][3] (c,k),
 * gqA[3][6], gdB[3][3], gqB[3][6].  Restates multipole_cgto and
 * multipole_grad_cgto, reference integrals.f90:1182-1391. */
typedef struct {
    double s[5][5], dA[3][5][5], qA[6][5][5], dB[3][5][5], qB[6][5][5];
    double gs[3][5][5], gdA[3][3][5][5], gqA[3][6][5][5], gdB[3][3][5][5], gqB[3][6][5][5];
} shellpair_t;

static void traceless(double q[6]) {
    double tr = 0.5 * (q[0] + q[2] + q[5]);
    q[0] = 1.5 * q[0] - tr;
    q[1] = 1.5 * q[1];
    q[2] = 1.5 * q[2] - tr;
    q[3] = 1.5 * q[3];
    q[4] = 1.5 * q[4];
    q[5] = 1.5 * q[5] - tr;
}

static const int QA[6] = {0, 0, 1, 0, 1, 2}; /* xx xy yy xz yz zz */
static const int QB[6] = {0, 1, 1, 2, 2, 2};

static void shell_pair(const cgto_t *cj, const cgto_t *ci, const double vec[3], double intcut,
                       int grad, shellpair_t *out) {
    init_trafo();
    const int lj = cj->l, li = ci->l;
    const int ncj = NCART[lj], nci = NCART[li];
    /* cartesian accumulators */
    double cs[6][6] = {{0}}, cdA[3][6][6] = {{{0}}}, cqA[6][6][6] = {{{0}}};
    double cdB[3][6][6] = {{{0}}}, cqB[6][6][6] = {{{0}}};
    double gs[3][6][6] = {{{0}}}, gdA[3][3][6][6] = {{{{0}}}}, gqA[3][6][6][6] = {{{{0}}}};
    double gdB[3][3][6][6] = {{{{0}}}}, gqB[3][6][6][6] = {{{{0}}}};
    const double r2 = vec[0] * vec[0] + vec[1] * vec[1] + vec[2] * vec[2];
    const double pi3 = pow(M_PI, 1.5);
    for (int ip = 0; ip < ci->nprim; ++ip) {
        for (int jp = 0; jp < cj->nprim; ++jp) {
            const double ai = ci->alpha[ip], aj = cj->alpha[jp];
            const double eta = ai + aj, oeta = 1.0 / eta;
            const double est = ai * aj * r2 * oeta;
            if (est > intcut) continue;
            const double cc = ci->coeff[ip] * cj->coeff[jp] * exp(-est) * pi3 * pow(oeta, 1.5);
            double pa[3], pb[3];
            for (int k = 0; k < 3; ++k) {
                /* A = R_B + vec;  P = (ai A + aj B)/eta */
                pa[k] = -vec[k] * aj * oeta; /* P - A */
                pb[k] = vec[k] * ai * oeta;  /* P - B */
            }
            for (int mi = 0; mi < nci; ++mi) {
                for (int mj = 0; mj < ncj; ++mj) {
                    /* 1-d factors: [dir][e] about A and about B, and A-derivatives */
                    double fA[3][3], fB[3][3], gA[3][3], gB[3][3];
                    for (int k = 0; k < 3; ++k) {
                        const int a = CEXP[li][mi][k], b = CEXP[lj][mj][k];
                        for (int e = 0; e < 3; ++e) {
                            fA[k][e] = mom1d(a, b, pa[k], pb[k], pa[k], e, eta);
                            fB[k][e] = mom1d(a, b, pa[k], pb[k], pb[k], e, eta);
                            if (grad) {
                                /* d/dA of (x-A)^a exp(-ai (x-A)^2) */
                                gA[k][e] = 2 * ai * mom1d(a + 1, b, pa[k], pb[k], pa[k], e, eta)
                                           - a * mom1d(a - 1, b, pa[k], pb[k], pa[k], e, eta);
                                gB[k][e] = 2 * ai * mom1d(a + 1, b, pa[k], pb[k], pb[k], e, eta)
                                           - a * mom1d(a - 1, b, pa[k], pb[k], pb[k], e, eta);
                            }
                        }
                    }
                    /* value of a product of 1-d factors with moment exponents ex[3] */
#define PROD(F, e0, e1, e2) (F[0][e0] * F[1][e1] * F[2][e2])
                    cs[mj][mi] += cc * PROD(fA, 0, 0, 0);
                    for (int k = 0; k < 3; ++k) {
                        int ex[3] = {0, 0, 0};
                        ex[k] = 1;
                        cdA[k][mj][mi] += cc * PROD(fA, ex[0], ex[1], ex[2]);
                        cdB[k][mj][mi] += cc * PROD(fB, ex[0], ex[1], ex[2]);
                    }
                    for (int q = 0; q < 6; ++q) {
                        int ex[3] = {0, 0, 0};
                        ex[QA[q]] += 1;
                        ex[QB[q]] += 1;
                        cqA[q][mj][mi] += cc * PROD(fA, ex[0], ex[1], ex[2]);
                        cqB[q][mj][mi] += cc * PROD(fB, ex[0], ex[1], ex[2]);
                    }
                    if (grad) {
                        for (int c = 0; c < 3; ++c) {
                            /* derivative acts on direction c only (function i) */
                            double FA[3][3], FB[3][3];
                            memcpy(FA, fA, sizeof(FA));
                            memcpy(FB, fB, sizeof(FB));
                            for (int e = 0; e < 3; ++e) {
                                FA[c][e] = gA[c][e];
                                FB[c][e] = gB[c][e];
                            }
                            gs[c][mj][mi] += cc * PROD(FA, 0, 0, 0);
                            for (int k = 0; k < 3; ++k) {
                                int ex[3] = {0, 0, 0};
                                ex[k] = 1;
                                /* operator on A moves with A: extra -delta_ck S */
                                double v = PROD(FA, ex[0], ex[1], ex[2]);
                                if (c == k) v -= PROD(fA, 0, 0, 0);
                                gdA[c][k][mj][mi] += cc * v;
                                gdB[c][k][mj][mi] += cc * PROD(FB, ex[0], ex[1], ex[2]);
                            }
                            for (int q = 0; q < 6; ++q) {
                                int ex[3] = {0, 0, 0};
                                ex[QA[q]] += 1;
                                ex[QB[q]] += 1;
                                double v = PROD(FA, ex[0], ex[1], ex[2]);
                                /* d/dA_c (x_a - A_a)(x_b - A_b): -delta_ac M_b - delta_bc M_a */
                                if (QA[q] == c) {
                                    int e2[3] = {0, 0, 0};
                                    e2[QB[q]] = 1;
                                    v -= PROD(fA, e2[0], e2[1], e2[2]);
                                }
                                if (QB[q] == c) {
                                    int e2[3] = {0, 0, 0};
                                    e2[QA[q]] = 1;
                                    v -= PROD(fA, e2[0], e2[1], e2[2]);
                                }
                                gqA[c][q][mj][mi] += cc * v;
                                gqB[c][q][mj][mi] += cc * PROD(FB, ex[0], ex[1], ex[2]);
                            }
                        }
                    }
#undef PROD
                }
            }
        }
    }
    /* traceless quadrupoles (cartesian, before the spherical transform; linear) */
    for (int mj = 0; mj < ncj; ++mj)
        for (int mi = 0; mi < nci; ++mi) {
            double t[6];
            for (int q = 0; q < 6; ++q) t[q] = cqA[q][mj][mi];
            traceless(t);
            for (int q = 0; q < 6; ++q) cqA[q][mj][mi] = t[q];
            for (int q = 0; q < 6; ++q) t[q] = cqB[q][mj][mi];
            traceless(t);
            for (int q = 0; q < 6; ++q) cqB[q][mj][mi] = t[q];
            if (grad)
                for (int c = 0; c < 3; ++c) {
                    for (int q = 0; q < 6; ++q) t[q] = gqA[c][q][mj][mi];
                    traceless(t);
                    for (int q = 0; q < 6; ++q) gqA[c][q][mj][mi] = t[q];
                    for (int q = 0; q < 6; ++q) t[q] = gqB[c][q][mj][mi];
                    traceless(t);
                    for (int q = 0; q < 6; ++q) gqB[c][q][mj][mi] = t[q];
                }
        }
    /* spherical transform of both indices */
    const int nsj = NSPH[lj], nsi = NSPH[li];
#define TRANS(dst, src)                                                              \
    for (int sj = 0; sj < nsj; ++sj)                                                 \
        for (int si = 0; si < nsi; ++si) {                                           \
            double acc = 0.0;                                                        \
            for (int mj = 0; mj < ncj; ++mj)                                         \
                for (int mi = 0; mi < nci; ++mi)                                     \
                    acc += TRAFO[lj][sj][mj] * TRAFO[li][si][mi] * (src)[mj][mi];    \
            (dst)[sj][si] = acc;                                                     \
        }
    TRANS(out->s, cs);
    for (int k = 0; k < 3; ++k) {
        TRANS(out->dA[k], cdA[k]);
        TRANS(out->dB[k], cdB[k]);
    }
    for (int q = 0; q < 6; ++q) {
        TRANS(out->qA[q], cqA[q]);
        TRANS(out->qB[q], cqB[q]);
    }
    if (grad) {
        for (int c = 0; c < 3; ++c) {
            TRANS(out->gs[c], gs[c]);
            for (int k = 0; k < 3; ++k) {
                TRANS(out->gdA[c][k], gdA[c][k]);
                TRANS(out->gdB[c][k], gdB[c][k]);
            }
            for (int q = 0; q < 6; ++q) {
                TRANS(out->gqA[c][q], gqA[c][q]);
                TRANS(out->gqB[c][q], gqB[c][q]);
            }
        }
    }
#undef TRANS
}

/* ------------------------------------------------------------------ */
/* Basis description passed from Python                                */
/* ------------------------------------------------------------------ */
typedef struct {
    int nat, nsh, nao;
    const double *xyz;      /* [nat][3] */
    const int *sh_atom;     /* [nsh] */
    const int *sh_l;        /* [nsh] */
    const int *sh_nprim;    /* [nsh] */
    const double *sh_alpha; /* [nsh][MAXG] */
    const double *sh_coeff; /* [nsh][MAXG] */
    const int *sh_ao;       /* [nsh] first AO */
    const int *at_sh;       /* [nat+1] shell offsets */
} basis_t;

static void get_cgto(const basis_t *b, int ish, cgto_t *c) {
    c->l = b->sh_l[ish];
    c->nprim = b->sh_nprim[ish];
    for (int p = 0; p < MAXG; ++p) {
        c->alpha[p] = b->sh_alpha[ish * MAXG + p];
        c->coeff[p] = b->sh_coeff[ish * MAXG + p];
    }
}

/* Single shell pair entry point (used by the integral unit tests).
 * out arrays: s[5*5], dA[3*25], qA[6*25], dB, qB, gs[3*25], gdA[9*25], gqA[18*25], gdB, gqB */
void orc_shell_pair(int lj, int nj, const double *aj, const double *cj, int li, int ni,
                    const double *ai, const double *ci, const double *vec, double intcut,
                    int grad, double *out) {
    cgto_t gj = {lj, nj}, gi = {li, ni};
    for (int p = 0; p < nj; ++p) { gj.alpha[p] = aj[p]; gj.coeff[p] = cj[p]; }
    for (int p = 0; p < ni; ++p) { gi.alpha[p] = ai[p]; gi.coeff[p] = ci[p]; }
    shellpair_t *sp = (shellpair_t *)calloc(1, sizeof(shellpair_t));
    shell_pair(&gj, &gi, vec, intcut, grad, sp);
    memcpy(out, sp, sizeof(shellpair_t));
    free(sp);
}
int orc_shellpair_size(void) { return (int)(sizeof(shellpair_t) / sizeof(double)); }

/* H0 build: reference src/tblite/xtb/h0.f90:220-429 (get_hamiltonian).
 * hscale[nsh_j][nsh_i] is not materialised: it is rebuilt from per-shell data
 * as in src/tblite/xtb/gfn2.f90:767-797 (get_hscale):
 *   hscale = (2 sqrt(zi zj)/(zi+zj))^wexp * kshell(lj, li) * (1 + enscale (EN_i-EN_j)^2)
 * shpoly[nsh], sh_zeta[nsh], at_en[nat], at_rad[nat], selfenergy[nsh].
 * hspair[nsh][nsh] (optional): a precomputed shell-pair scale that replaces the GFN2 formula
 * (GFN1: valence/polarisation shells and element-pair factors, xtb/gfn1.f90:797-828). */
void orc_build_h0(const basis_t *b, const double *selfenergy, const double *shpoly,
                  const double *sh_zeta, const double *at_en, const double *at_rad,
                  const double *kshell /*[5][5]*/, double wexp, double enscale, double intcut,
                  double cutoff, double *S, double *D, double *Q, double *H,
                  const double *hspair) {
    const int nshl = b->nsh;
    const int n = b->nao;
    const size_t nn = (size_t)n * n;
    memset(S, 0, nn * sizeof(double));
    memset(H, 0, nn * sizeof(double));
    memset(D, 0, 3 * nn * sizeof(double));
    memset(Q, 0, 6 * nn * sizeof(double));
    const double cut2 = cutoff * cutoff;
#pragma omp parallel for schedule(dynamic)
    for (int iat = 0; iat < b->nat; ++iat) {
        shellpair_t *sp = (shellpair_t *)malloc(sizeof(shellpair_t));
        for (int jat = 0; jat <= iat; ++jat) {
            double vec[3];
            for (int k = 0; k < 3; ++k) vec[k] = b->xyz[3 * iat + k] - b->xyz[3 * jat + k];
            const double r2 = vec[0] * vec[0] + vec[1] * vec[1] + vec[2] * vec[2];
            if (iat != jat && (r2 > cut2 || r2 < 2.220446049250313e-16)) continue;
            const double rr = iat != jat ? sqrt(sqrt(r2) / (at_rad[iat] + at_rad[jat])) : 0.0;
            for (int ish = b->at_sh[iat]; ish < b->at_sh[iat + 1]; ++ish) {
                cgto_t ci;
                get_cgto(b, ish, &ci);
                for (int jsh = b->at_sh[jat]; jsh < b->at_sh[jat + 1]; ++jsh) {
                    cgto_t cj;
                    get_cgto(b, jsh, &cj);
                    shell_pair(&cj, &ci, vec, intcut, 0, sp);
                    double hij;
                    if (iat != jat) {
                        const double zi = sh_zeta[ish], zj = sh_zeta[jsh];
                        const double zij = pow(2 * sqrt(zi * zj) / (zi + zj), wexp);
                        const double den = (at_en[iat] - at_en[jat]) * (at_en[iat] - at_en[jat]);
                        const double hs = hspair ? hspair[(size_t)jsh * nshl + ish]
                                                 : zij * kshell[cj.l * 5 + ci.l] * (1.0 + enscale * den);
                        const double poly = (1.0 + shpoly[ish] * rr) * (1.0 + shpoly[jsh] * rr);
                        hij = 0.5 * (selfenergy[ish] + selfenergy[jsh]) * hs * poly;
                    } else {
                        hij = 0.5 * (selfenergy[ish] + selfenergy[jsh]);
                    }
                    const int io = b->sh_ao[ish], jo = b->sh_ao[jsh];
                    for (int mi = 0; mi < NSPH[ci.l]; ++mi) {
                        for (int mj = 0; mj < NSPH[cj.l]; ++mj) {
                            const size_t ji = (size_t)(jo + mj) * n + (io + mi);
                            const size_t ij = (size_t)(io + mi) * n + (jo + mj);
                            const double s = sp->s[mj][mi];
                            S[ji] = s;
                            H[ji] = s * hij;
                            for (int k = 0; k < 3; ++k) D[k * nn + ji] = sp->dA[k][mj][mi];
                            for (int q = 0; q < 6; ++q) Q[q * nn + ji] = sp->qA[q][mj][mi];
                            if (iat != jat) {
                                S[ij] = s;
                                H[ij] = s * hij;
                                for (int k = 0; k < 3; ++k) D[k * nn + ij] = sp->dB[k][mj][mi];
                                for (int q = 0; q < 6; ++q) Q[q * nn + ij] = sp->qB[q][mj][mi];
                            }
                        }
                    }
                }
            }
        }
        free(sp);
    }
}

/* H0 gradient: reference src/tblite/xtb/h0.f90:432-666.
 * P, W: [n][n] (total density, energy weighted density), vao[n], vdp[nat][3],
 * vqp[nat][6], dsedcn[nsh].  Accumulates gradient[nat][3], sigma[3][3], dEdcn[nat]. */
void orc_h0_gradient(const basis_t *b, const double *selfenergy, const double *dsedcn,
                     const double *shpoly, const double *sh_zeta, const double *at_en,
                     const double *at_rad, const double *kshell, double wexp, double enscale,
                     double intcut, double cutoff, const double *P, const double *W,
                     const double *vao, const double *vdp, const double *vqp, double *gradient,
                     double *sigma, double *dEdcn, const double *hspair) {
    const int n = b->nao, nat = b->nat, nshl = b->nsh;
    const double cut2 = cutoff * cutoff;
    double *g_acc = (double *)calloc((size_t)nat * 3, sizeof(double));
    double *c_acc = (double *)calloc((size_t)nat, sizeof(double));
    double s_acc[9] = {0};
#pragma omp parallel
    {
        double *g_loc = (double *)calloc((size_t)nat * 3, sizeof(double));
        double *c_loc = (double *)calloc((size_t)nat, sizeof(double));
        double s_loc[9] = {0};
        shellpair_t *sp = (shellpair_t *)malloc(sizeof(shellpair_t));
#pragma omp for schedule(dynamic)
        for (int iat = 0; iat < nat; ++iat) {
            for (int jat = 0; jat < iat; ++jat) {
                double vec[3];
                for (int k = 0; k < 3; ++k) vec[k] = b->xyz[3 * iat + k] - b->xyz[3 * jat + k];
                const double r2 = vec[0] * vec[0] + vec[1] * vec[1] + vec[2] * vec[2];
                if (r2 > cut2 || r2 < 2.220446049250313e-16) continue;
                const double rr = sqrt(sqrt(r2) / (at_rad[iat] + at_rad[jat]));
                double dG[3] = {0, 0, 0}, dcni = 0, dcnj = 0;
                for (int ish = b->at_sh[iat]; ish < b->at_sh[iat + 1]; ++ish) {
                    cgto_t ci;
                    get_cgto(b, ish, &ci);
                    const double polyi = 1.0 + shpoly[ish] * rr;
                    for (int jsh = b->at_sh[jat]; jsh < b->at_sh[jat + 1]; ++jsh) {
                        cgto_t cj;
                        get_cgto(b, jsh, &cj);
                        shell_pair(&cj, &ci, vec, intcut, 1, sp);
                        const double polyj = 1.0 + shpoly[jsh] * rr;
                        const double poly = polyi * polyj;
                        const double dpoly = (polyi * shpoly[jsh] + polyj * shpoly[ish]) * 0.5 * rr / r2;
                        double dsv[3];
                        for (int k = 0; k < 3; ++k) dsv[k] = dpoly / poly * vec[k];
                        const double zi = sh_zeta[ish], zj = sh_zeta[jsh];
                        const double zij = pow(2 * sqrt(zi * zj) / (zi + zj), wexp);
                        const double den = (at_en[iat] - at_en[jat]) * (at_en[iat] - at_en[jat]);
                        const double hs = (hspair ? hspair[(size_t)jsh * nshl + ish]
                                                  : zij * kshell[cj.l * 5 + ci.l] * (1.0 + enscale * den)) * poly;
                        const double hij = 0.5 * (selfenergy[ish] + selfenergy[jsh]) * hs;
                        const double dhdcni = dsedcn[ish] * hs, dhdcnj = dsedcn[jsh] * hs;
                        const int io = b->sh_ao[ish], jo = b->sh_ao[jsh];
                        for (int mi = 0; mi < NSPH[ci.l]; ++mi) {
                            for (int mj = 0; mj < NSPH[cj.l]; ++mj) {
                                const int ia = io + mi, ja = jo + mj;
                                const double pij = P[(size_t)ja * n + ia];
                                const double wij = W[(size_t)ja * n + ia];
                                const double s = sp->s[mj][mi];
                                const double sval = -pij * (vao[ja] + vao[ia]) + 2 * pij * hij - 2 * wij;
                                for (int c = 0; c < 3; ++c) {
                                    double g = sval * sp->gs[c][mj][mi] + 2 * pij * hij * s * dsv[c];
                                    double vd = 0.0;
                                    for (int k = 0; k < 3; ++k)
                                        vd += sp->gdA[c][k][mj][mi] * vdp[3 * iat + k]
                                              + sp->gdB[c][k][mj][mi] * vdp[3 * jat + k];
                                    for (int q = 0; q < 6; ++q)
                                        vd += sp->gqA[c][q][mj][mi] * vqp[6 * iat + q]
                                              + sp->gqB[c][q][mj][mi] * vqp[6 * jat + q];
                                    dG[c] += g - pij * vd;
                                }
                                dcni += dhdcni * pij * s;
                                dcnj += dhdcnj * pij * s;
                            }
                        }
                    }
                }
                c_loc[iat] += dcni;
                c_loc[jat] += dcnj;
                for (int c = 0; c < 3; ++c) {
                    g_loc[3 * iat + c] += dG[c];
                    g_loc[3 * jat + c] -= dG[c];
                }
                for (int a = 0; a < 3; ++a)
                    for (int c = 0; c < 3; ++c)
                        s_loc[3 * a + c] += 0.5 * (vec[a] * dG[c] + dG[a] * vec[c]);
            }
            /* on-site CN derivative of the diagonal levels */
            for (int ish = b->at_sh[iat]; ish < b->at_sh[iat + 1]; ++ish) {
                const int io = b->sh_ao[ish];
                for (int mi = 0; mi < NSPH[b->sh_l[ish]]; ++mi)
                    c_loc[iat] += dsedcn[ish] * P[(size_t)(io + mi) * n + io + mi];
            }
        }
        free(sp);
#pragma omp critical
        {
            for (int i = 0; i < 3 * nat; ++i) g_acc[i] += g_loc[i];
            for (int i = 0; i < nat; ++i) c_acc[i] += c_loc[i];
            for (int i = 0; i < 9; ++i) s_acc[i] += s_loc[i];
        }
        free(g_loc);
        free(c_loc);
    }
    for (int i = 0; i < 3 * nat; ++i) gradient[i] += g_acc[i];
    for (int i = 0; i < nat; ++i) dEdcn[i] += c_acc[i];
    for (int i = 0; i < 9; ++i) sigma[i] += s_acc[i];
    free(g_acc);
    free(c_acc);
}

/* ------------------------------------------------------------------ */
/* Coordination number, double-exponential counting function           */
/* count(r) = f(ka, r0/r) * f(kb, (r0 + rshift)/r), f(k,x) = 1/(1+exp(-k(x-1)))
 * with r0 = rcov_A + rcov_B.  Used for the GFN2 self-energy shift
 * (reference xtb/singlepoint.f90:218-225) and the AES radii (coulomb/multipole.f90:181).
 * The counting function belongs to mctc-lib (not part of the reference tree);
 * its constants come in through the element-data pack.                 */
/* ------------------------------------------------------------------ */
static void dexp_count(double r, double r0, double ka, double kb, double rshift, double *cnt,
                       double *dcnt) {
    const double e1 = exp(-ka * (r0 / r - 1.0));
    const double e2 = exp(-kb * ((r0 + rshift) / r - 1.0));
    const double f1 = 1.0 / (1.0 + e1), f2 = 1.0 / (1.0 + e2);
    *cnt = f1 * f2;
    /* d f/dr = -f^2 * e * k * x / r  (x = r0/r) */
    const double d1 = -f1 * f1 * e1 * ka * r0 / (r * r);
    const double d2 = -f2 * f2 * e2 * kb * (r0 + rshift) / (r * r);
    *dcnt = d1 * f2 + f1 * d2;
}

void orc_cn_dexp(int nat, const double *xyz, const double *rcov, double ka, double kb,
                 double rshift, double cutoff, double *cn) {
    const double cut2 = cutoff * cutoff;
    memset(cn, 0, nat * sizeof(double));
    for (int i = 0; i < nat; ++i)
        for (int j = 0; j < i; ++j) {
            double v[3], r2 = 0;
            for (int k = 0; k < 3; ++k) { v[k] = xyz[3 * i + k] - xyz[3 * j + k]; r2 += v[k] * v[k]; }
            if (r2 > cut2 || r2 < 1e-12) continue;
            double c, dc;
            dexp_count(sqrt(r2), rcov[i] + rcov[j], ka, kb, rshift, &c, &dc);
            cn[i] += c;
            cn[j] += c;
        }
}

/* gradient += dCN/dR^T dEdcn (the reference materialises dcndr(3,N,N) and calls gemv,
 * xtb/singlepoint.f90:374-379; here the contraction is done pair by pair). */
void orc_cn_dexp_grad(int nat, const double *xyz, const double *rcov, double ka, double kb,
                      double rshift, double cutoff, const double *dEdcn, double *gradient,
                      double *sigma) {
    const double cut2 = cutoff * cutoff;
    for (int i = 0; i < nat; ++i)
        for (int j = 0; j < i; ++j) {
            double v[3], r2 = 0;
            for (int k = 0; k < 3; ++k) { v[k] = xyz[3 * i + k] - xyz[3 * j + k]; r2 += v[k] * v[k]; }
            if (r2 > cut2 || r2 < 1e-12) continue;
            const double r = sqrt(r2);
            double c, dc;
            dexp_count(r, rcov[i] + rcov[j], ka, kb, rshift, &c, &dc);
            const double f = (dEdcn[i] + dEdcn[j]) * dc / r;
            for (int k = 0; k < 3; ++k) {
                gradient[3 * i + k] += f * v[k];
                gradient[3 * j + k] -= f * v[k];
            }
            for (int a = 0; a < 3; ++a)
                for (int b2 = 0; b2 < 3; ++b2) sigma[3 * a + b2] += f * v[a] * v[b2];
        }
}

/* ------------------------------------------------------------------ */
/* Isotropic electrostatics, reference coulomb/charge/effective.f90:238-286 (get_amat_0d)
 * gamma_ab = 1/(R^g + eta_ab^-g)^(1/g) with eta_ab = average of shell hardnesses.
 * hub[nsh_total] shell hardness per shell; avg: 0 arithmetic (GFN2), 1 harmonic (GFN1). */
/* ------------------------------------------------------------------ */
static double average(double a, double b, int kind) {
    if (kind == 0) return 0.5 * (a + b);
    if (kind == 1) return 2.0 / (1.0 / a + 1.0 / b);
    return sqrt(a * b);
}

void orc_gamma(int nat, const double *xyz, const int *at_sh, const double *hub, double gexp,
               int avg, double *amat /*[nsh][nsh]*/) {
    const int nsh = at_sh[nat];
    memset(amat, 0, (size_t)nsh * nsh * sizeof(double));
    for (int i = 0; i < nat; ++i) {
        for (int j = 0; j < i; ++j) {
            double r2 = 0;
            for (int k = 0; k < 3; ++k) {
                double d = xyz[3 * j + k] - xyz[3 * i + k];
                r2 += d * d;
            }
            const double r1 = sqrt(r2), r1g = pow(r1, gexp);
            for (int is = at_sh[i]; is < at_sh[i + 1]; ++is)
                for (int js = at_sh[j]; js < at_sh[j + 1]; ++js) {
                    const double gam = average(hub[is], hub[js], avg);
                    const double t = 1.0 / pow(r1g + pow(gam, -gexp), 1.0 / gexp);
                    amat[(size_t)js * nsh + is] += t;
                    amat[(size_t)is * nsh + js] += t;
                }
        }
        for (int is = at_sh[i]; is < at_sh[i + 1]; ++is)
            for (int js = at_sh[i]; js < at_sh[i + 1]; ++js)
                amat[(size_t)js * nsh + is] = average(hub[is], hub[js], avg);
    }
}

/* gradient of 1/2 q^T gamma q, reference effective.f90:487-556 + charge/type.f90:266-294 */
void orc_gamma_grad(int nat, const double *xyz, const int *at_sh, const double *hub, double gexp,
                    int avg, const double *qsh, double *gradient, double *sigma) {
    for (int i = 0; i < nat; ++i)
        for (int j = 0; j < i; ++j) {
            double v[3], r2 = 0;
            for (int k = 0; k < 3; ++k) { v[k] = xyz[3 * i + k] - xyz[3 * j + k]; r2 += v[k] * v[k]; }
            const double r1 = sqrt(r2);
            double f = 0.0;
            for (int is = at_sh[i]; is < at_sh[i + 1]; ++is)
                for (int js = at_sh[j]; js < at_sh[j + 1]; ++js) {
                    const double gam = average(hub[is], hub[js], avg);
                    double d = 1.0 / (pow(r1, gexp) + pow(gam, -gexp));
                    d = -pow(r1, gexp - 2.0) * d * pow(d, 1.0 / gexp);
                    f += d * qsh[is] * qsh[js];
                }
            for (int k = 0; k < 3; ++k) {
                gradient[3 * i + k] += f * v[k];
                gradient[3 * j + k] -= f * v[k];
            }
            for (int a = 0; a < 3; ++a)
                for (int b2 = 0; b2 < 3; ++b2) sigma[3 * a + b2] += f * v[a] * v[b2];
        }
}

/* ------------------------------------------------------------------ */
/* Anisotropic electrostatics (AES), reference coulomb/multipole.f90:488-535
 * amat_sd[i][j][3], amat_dd[i][j][3][3], amat_sq[i][j][6]  (first index = iat,
 * i.e. the reference's amat(:, jat, iat) stored at [iat][jat]). */
/* ------------------------------------------------------------------ */
void orc_aes_matrices(int nat, const double *xyz, const double *mrad, double kdmp3, double kdmp5,
                      double *asd, double *add, double *asq) {
    memset(asd, 0, (size_t)nat * nat * 3 * sizeof(double));
    memset(add, 0, (size_t)nat * nat * 9 * sizeof(double));
    memset(asq, 0, (size_t)nat * nat * 6 * sizeof(double));
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nat; ++i)
        for (int j = 0; j < nat; ++j) {
            if (i == j) continue;
            double v[3];
            for (int k = 0; k < 3; ++k) v[k] = xyz[3 * i + k] - xyz[3 * j + k];
            const double r1 = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
            const double g1 = 1.0 / r1, g3 = g1 * g1 * g1, g5 = g3 * g1 * g1;
            const double rr = 0.5 * (mrad[j] + mrad[i]) * g1;
            const double f3 = 1.0 / (1.0 + 6.0 * pow(rr, kdmp3));
            const double f5 = 1.0 / (1.0 + 6.0 * pow(rr, kdmp5));
            const size_t ij = (size_t)i * nat + j;
            for (int k = 0; k < 3; ++k) asd[ij * 3 + k] = v[k] * g3 * f3;
            for (int a = 0; a < 3; ++a)
                for (int c = 0; c < 3; ++c)
                    add[ij * 9 + 3 * a + c] = (a == c ? g3 * f5 : 0.0) - v[a] * v[c] * 3 * g5 * f5;
            asq[ij * 6 + 0] = v[0] * v[0] * g5 * f5;
            asq[ij * 6 + 1] = 2 * v[0] * v[1] * g5 * f5;
            asq[ij * 6 + 2] = v[1] * v[1] * g5 * f5;
            asq[ij * 6 + 3] = 2 * v[0] * v[2] * g5 * f5;
            asq[ij * 6 + 4] = 2 * v[1] * v[2] * g5 * f5;
            asq[ij * 6 + 5] = v[2] * v[2] * g5 * f5;
        }
}

/* AES gradient at fixed moments, reference multipole.f90:746-852 (get_multipole_gradient_0d).
 * dEdr[nat] accumulates the derivative w.r.t. the damping radii. */
void orc_aes_grad(int nat, const double *xyz, const double *mrad, double kdmp3, double kdmp5,
                  const double *qat, const double *dpat, const double *qpat, double *dEdr,
                  double *gradient, double *sigma) {
    for (int i = 0; i < nat; ++i)
        for (int j = 0; j < i; ++j) {
            const double rr = 0.5 * (mrad[i] + mrad[j]);
            double v[3];
            for (int k = 0; k < 3; ++k) v[k] = xyz[3 * j + k] - xyz[3 * i + k];
            const double r2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2], r1 = sqrt(r2);
            const double g1 = 1.0 / r1, g3 = g1 * g1 * g1, g5 = g3 * g1 * g1, g7 = g5 * g1 * g1;
            const double f3 = 1.0 / (1.0 + 6.0 * pow(rr * g1, kdmp3));
            const double d3 = -3 * g5 * f3 - kdmp3 * f3 * (f3 - 1.0) * g5;
            const double f5 = 1.0 / (1.0 + 6.0 * pow(rr * g1, kdmp5));
            const double d5 = -5 * f5 - kdmp5 * (f5 * f5 - f5);
            const double *di = dpat + 3 * i, *dj = dpat + 3 * j;
            const double *qi = qpat + 6 * i, *qj = qpat + 6 * j;
            double dG[3], fddr;
            /* charge-dipole */
            const double dpiqj = (v[0] * di[0] + v[1] * di[1] + v[2] * di[2]) * qat[j];
            const double qidpj = (v[0] * dj[0] + v[1] * dj[1] + v[2] * dj[2]) * qat[i];
            fddr = 3.0 * (dpiqj - qidpj) * kdmp3 * f3 * g3 * (f3 / rr) * pow(rr * g1, kdmp3);
            for (int k = 0; k < 3; ++k)
                dG[k] = -d3 * v[k] * (dpiqj - qidpj) + f3 * g3 * (qat[i] * dj[k] - qat[j] * di[k]);
            /* dipole-dipole */
            const double dpidpj = di[0] * dj[0] + di[1] * dj[1] + di[2] * dj[2];
            const double dpiv = di[0] * v[0] + di[1] * v[1] + di[2] * v[2];
            const double dpjv = dj[0] * v[0] + dj[1] * v[1] + dj[2] * v[2];
            const double edd = dpidpj * r2 - 3 * dpjv * dpiv;
            double fddr2 = 3.0 * edd * kdmp5 * f5 * g5 * (f5 / rr) * pow(rr * g1, kdmp5);
            double dG2[3];
            for (int k = 0; k < 3; ++k)
                dG2[k] = -2.0 * f5 * g5 * dpidpj * v[k] + 3.0 * f5 * g5 * (dpiv * dj[k] + dpjv * di[k])
                         - edd * d5 * g7 * v[k];
            /* charge-quadrupole */
            const double eq = 2 * (qat[j] * qi[1] + qj[1] * qat[i]) * v[0] * v[1]
                              + 2 * (qat[j] * qi[3] + qj[3] * qat[i]) * v[0] * v[2]
                              + 2 * (qat[j] * qi[4] + qj[4] * qat[i]) * v[1] * v[2]
                              + (qat[j] * qi[0] + qj[0] * qat[i]) * v[0] * v[0]
                              + (qat[j] * qi[2] + qj[2] * qat[i]) * v[1] * v[1]
                              + (qat[j] * qi[5] + qj[5] * qat[i]) * v[2] * v[2];
            double fddr3 = eq * 3.0 * kdmp5 * f5 * g5 * f5 / rr * pow(rr * g1, kdmp5);
            double qjv[3] = {v[0] * qj[0] + v[1] * qj[1] + v[2] * qj[3],
                             v[0] * qj[1] + v[1] * qj[2] + v[2] * qj[4],
                             v[0] * qj[3] + v[1] * qj[4] + v[2] * qj[5]};
            double qiv[3] = {v[0] * qi[0] + v[1] * qi[1] + v[2] * qi[3],
                             v[0] * qi[1] + v[1] * qi[2] + v[2] * qi[4],
                             v[0] * qi[3] + v[1] * qi[4] + v[2] * qi[5]};
            double dG3[3];
            for (int k = 0; k < 3; ++k)
                dG3[k] = -eq * d5 * g7 * v[k] - 2.0 * f5 * g5 * qat[i] * qjv[k]
                         - 2.0 * f5 * g5 * qat[j] * qiv[k];
            dEdr[i] += fddr + fddr2 + fddr3;
            dEdr[j] += fddr + fddr2 + fddr3;
            for (int k = 0; k < 3; ++k) {
                const double g = dG[k] + dG2[k] + dG3[k];
                gradient[3 * i + k] += g;
                gradient[3 * j + k] -= g;
            }
            for (int a = 0; a < 3; ++a)
                for (int c = 0; c < 3; ++c) {
                    const double ga = dG[a] + dG2[a] + dG3[a], gc = dG[c] + dG2[c] + dG3[c];
                    sigma[3 * a + c] -= 0.5 * (v[a] * gc + ga * v[c]);
                }
        }
}

/* ------------------------------------------------------------------ */
/* Repulsion, reference repulsion/effective.f90:187-247                */
/* alpha_ij = sqrt(a_i a_j), zeff_ij = z_i z_j, kexp 1.5 (1.0 for H/He pairs) */
/* ------------------------------------------------------------------ */
void orc_repulsion(int nat, const double *xyz, const int *num, const double *alpha,
                   const double *zeff, double kexp, double kexp_light, double rexp, double cutoff,
                   double *energies, double *gradient, double *sigma) {
    const double cut2 = cutoff * cutoff;
    for (int i = 0; i < nat; ++i)
        for (int j = 0; j < i; ++j) {
            double v[3], r2 = 0;
            for (int k = 0; k < 3; ++k) { v[k] = xyz[3 * i + k] - xyz[3 * j + k]; r2 += v[k] * v[k]; }
            if (r2 > cut2 || r2 < 1e-12) continue;
            const double r1 = sqrt(r2);
            const double ke = (num[i] > 2 || num[j] > 2) ? kexp : kexp_light;
            const double a = sqrt(alpha[i] * alpha[j]), z = zeff[i] * zeff[j];
            const double r1k = pow(r1, ke), exa = exp(-a * r1k), r1r = pow(r1, rexp);
            const double dE = z * exa / r1r;
            energies[i] += 0.5 * dE;
            energies[j] += 0.5 * dE;
            if (gradient) {
                const double f = -(a * r1k * ke + rexp) * dE / r2;
                for (int k = 0; k < 3; ++k) {
                    gradient[3 * i + k] += f * v[k];
                    gradient[3 * j + k] -= f * v[k];
                }
                for (int a2 = 0; a2 < 3; ++a2)
                    for (int c = 0; c < 3; ++c) sigma[3 * a2 + c] += f * v[a2] * v[c];
            }
        }
}

/* ------------------------------------------------------------------ */
/* D4 dispersion.  The model is part of dftd4 (not in the reference tree); the
 * reference calls it from src/tblite/disp/d4.f90:105-474.  Restated from the
 * published D4 model: EN-weighted error-function coordination number,
 * Gaussian reference weights with charge scaling, rational (BJ) damping for the
 * two-body term, Axilrod-Teller-Muto three-body term with the same radii.
 * c6ref[ia][r][ib][s] is a table over the atoms' species (nsp species, MREF refs). */
/* ------------------------------------------------------------------ */
#define MREF 7

void orc_d4_cn(int nat, const double *xyz, const double *rcov, const double *en, double kn,
               double k4, double k5, double k6, double cutoff, const double *dEdcn, double *cn,
               double *gradient, double *sigma) {
    const double cut2 = cutoff * cutoff;
    if (cn) memset(cn, 0, nat * sizeof(double));
    for (int i = 0; i < nat; ++i)
        for (int j = 0; j < i; ++j) {
            double v[3], r2 = 0;
            for (int k = 0; k < 3; ++k) { v[k] = xyz[3 * i + k] - xyz[3 * j + k]; r2 += v[k] * v[k]; }
            if (r2 > cut2 || r2 < 1e-12) continue;
            const double r = sqrt(r2), rc = rcov[i] + rcov[j];
            const double den = k4 * exp(-pow(fabs(en[i] - en[j]) + k5, 2) / k6);
            const double arg = -kn * (r - rc) / rc;
            if (cn) {
                const double c = den * 0.5 * (1.0 + erf(arg));
                cn[i] += c;
                cn[j] += c;
            }
            if (gradient) {
                const double dc = -den * kn / rc * exp(-arg * arg) / sqrt(M_PI);
                const double f = (dEdcn[i] + dEdcn[j]) * dc / r;
                for (int k = 0; k < 3; ++k) {
                    gradient[3 * i + k] += f * v[k];
                    gradient[3 * j + k] -= f * v[k];
                }
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b) sigma[3 * a + b] += f * v[a] * v[b];
            }
        }
}

static double d4_pair_de(double r2, double rrij, double r0, double s6, double s8, double *ddedr) {
    const double r6 = r2 * r2 * r2, r8 = r6 * r2, r0_6 = pow(r0, 6), r0_8 = pow(r0, 8);
    const double t6 = 1.0 / (r6 + r0_6), t8 = 1.0 / (r8 + r0_8);
    if (ddedr) {
        const double r = sqrt(r2);
        *ddedr = s6 * 6.0 * r6 / r * t6 * t6 + s8 * rrij * 8.0 * r8 / r * t8 * t8;
    }
    return -(s6 * t6 + s8 * rrij * t8);
}

/* Two-body term with atom-wise weights gw[nat][MREF].
 * mode 0: u[nat][MREF] = sum_B dE_AB sum_s c6ref(rA,sB) gw_sB   (for potential / energy)
 * mode 1: gradient at fixed weights + dEdcn via dgwdcn (dE/dgw chain) */
void orc_d4_twobody(int nat, const double *xyz, const int *sp, int nsp, const double *c6ref,
                    const double *r4r2, double a1, double a2, double s6, double s8, double cutoff,
                    const double *gw, const double *dgwdcn, int mode, double *u, double *gradient,
                    double *sigma, double *dEdcn) {
    const double cut2 = cutoff * cutoff;
    const int ld = nsp * MREF;
    if (mode == 0) memset(u, 0, (size_t)nat * MREF * sizeof(double));
    for (int i = 0; i < nat; ++i)
        for (int j = 0; j < nat; ++j) {
            if (i == j) continue;
            double v[3], r2 = 0;
            for (int k = 0; k < 3; ++k) { v[k] = xyz[3 * i + k] - xyz[3 * j + k]; r2 += v[k] * v[k]; }
            if (r2 > cut2 || r2 < 1e-12) continue;
            const double rrij = 3.0 * r4r2[i] * r4r2[j];
            const double r0 = a1 * sqrt(rrij) + a2;
            double dd;
            const double de = d4_pair_de(r2, rrij, r0, s6, s8, &dd);
            const double *tab = c6ref + (size_t)sp[i] * MREF * ld + sp[j] * MREF;
            if (mode == 0) {
                for (int r = 0; r < MREF; ++r) {
                    double acc = 0.0;
                    for (int s = 0; s < MREF; ++s) acc += tab[(size_t)r * ld + s] * gw[j * MREF + s];
                    u[i * MREF + r] += de * acc;
                }
            } else if (j < i) {
                double c6 = 0.0, dc6i = 0.0, dc6j = 0.0;
                for (int r = 0; r < MREF; ++r)
                    for (int s = 0; s < MREF; ++s) {
                        const double t = tab[(size_t)r * ld + s];
                        c6 += gw[i * MREF + r] * gw[j * MREF + s] * t;
                        dc6i += dgwdcn[i * MREF + r] * gw[j * MREF + s] * t;
                        dc6j += gw[i * MREF + r] * dgwdcn[j * MREF + s] * t;
                    }
                dEdcn[i] += de * dc6i;
                dEdcn[j] += de * dc6j;
                const double f = dd * c6 / sqrt(r2);  /* d(de c6)/dR_i = dd c6 v/r */
                for (int k = 0; k < 3; ++k) {
                    gradient[3 * i + k] += f * v[k];
                    gradient[3 * j + k] -= f * v[k];
                }
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b) sigma[3 * a + b] += f * v[a] * v[b];
            }
        }
}

/* Three-body ATM term at fixed atomic C6 (c6[nat][nat]); energies split in thirds.
 * dEdc6[nat][nat] accumulates dE/dC6_ij (symmetric use) for the CN chain rule. */
void orc_d4_atm(int nat, const double *xyz, const double *c6, const double *r4r2, double a1,
                double a2, double s9, double alp, double cutoff, double *energies, double *dEdc6,
                double *gradient, double *sigma) {
    const double cut2 = cutoff * cutoff;
    for (int i = 0; i < nat; ++i)
        for (int j = 0; j < i; ++j) {
            double vij[3], r2ij = 0;
            for (int k = 0; k < 3; ++k) { vij[k] = xyz[3 * j + k] - xyz[3 * i + k]; r2ij += vij[k] * vij[k]; }
            if (r2ij > cut2 || r2ij < 1e-12) continue;
            const double r0ij = a1 * sqrt(3.0 * r4r2[i] * r4r2[j]) + a2;
            for (int l = 0; l < j; ++l) {
                double vik[3], vjk[3], r2ik = 0, r2jk = 0;
                for (int k = 0; k < 3; ++k) {
                    vik[k] = xyz[3 * l + k] - xyz[3 * i + k];
                    vjk[k] = xyz[3 * l + k] - xyz[3 * j + k];
                    r2ik += vik[k] * vik[k];
                    r2jk += vjk[k] * vjk[k];
                }
                if (r2ik > cut2 || r2jk > cut2 || r2ik < 1e-12 || r2jk < 1e-12) continue;
                const double r0ik = a1 * sqrt(3.0 * r4r2[i] * r4r2[l]) + a2;
                const double r0jk = a1 * sqrt(3.0 * r4r2[j] * r4r2[l]) + a2;
                const double c6ij = c6[i * nat + j], c6ik = c6[i * nat + l], c6jk = c6[j * nat + l];
                const double c9 = -s9 * sqrt(fabs(c6ij * c6ik * c6jk));
                const double r0 = r0ij * r0ik * r0jk;
                const double r2 = r2ij * r2ik * r2jk, r1 = sqrt(r2), r3 = r2 * r1, r5 = r3 * r2;
                const double fdmp = 1.0 / (1.0 + 6.0 * pow(r0 / r1, alp / 3.0));
                const double ang = 0.375 * (r2ij + r2jk - r2ik) * (r2ij - r2jk + r2ik)
                                       * (-r2ij + r2jk + r2ik) / r5 + 1.0 / r3;
                const double rr = ang * fdmp;
                const double dE = rr * c9;
                energies[i] += dE / 3.0;
                energies[j] += dE / 3.0;
                energies[l] += dE / 3.0;
                /* derivatives w.r.t. the three squared distances (x = r2ij etc.) */
                const double dfdmp = -2.0 * alp * pow(r0 / r1, alp / 3.0) * fdmp * fdmp;
                /* d ang / d r2ij (chain through the product terms), as in the published form */
                double dang[3];
                {
                    const double a = r2ij, b = r2jk, c = r2ik;
                    const double P = (a + b - c) * (a - b + c) * (-a + b + c);
                    const double dPa = (a - b + c) * (-a + b + c) + (a + b - c) * (-a + b + c)
                                       - (a + b - c) * (a - b + c);
                    const double dPb = (a - b + c) * (-a + b + c) - (a + b - c) * (-a + b + c)
                                       + (a + b - c) * (a - b + c);
                    const double dPc = -(a - b + c) * (-a + b + c) + (a + b - c) * (-a + b + c)
                                       + (a + b - c) * (a - b + c);
                    /* r5 = (abc)^(5/2), r3 = (abc)^(3/2) */
                    dang[0] = 0.375 * (dPa / r5 - 2.5 * P / (r5 * a)) - 1.5 / (r3 * a);
                    dang[1] = 0.375 * (dPb / r5 - 2.5 * P / (r5 * b)) - 1.5 / (r3 * b);
                    dang[2] = 0.375 * (dPc / r5 - 2.5 * P / (r5 * c)) - 1.5 / (r3 * c);
                }
                /* d fdmp / d r2x = dfdmp/6 * (-1/(2 r2x)) ... fdmp depends on r1 = sqrt(abc) */
                const double dfd[3] = {dfdmp / 6.0 * (-0.5 / r2ij) * -1.0, 0, 0};
                (void)dfd;
                /* fdmp = 1/(1+6 t), t = (r0/r1)^(alp/3); dt/d r2x = -(alp/6) t / r2x */
                const double t = pow(r0 / r1, alp / 3.0);
                const double dfdt = -6.0 * fdmp * fdmp;
                const double dx[3] = {r2ij, r2jk, r2ik};
                double dEd[3];
                for (int q = 0; q < 3; ++q) {
                    const double dtdx = -(alp / 6.0) * t / dx[q];
                    dEd[q] = c9 * (dang[q] * fdmp + ang * dfdt * dtdx);
                }
                /* gradient: d r2ij / dR_i = -2 vij (vij = R_j - R_i) */
                for (int k = 0; k < 3; ++k) {
                    const double gij = 2.0 * dEd[0] * vij[k], gjk = 2.0 * dEd[1] * vjk[k],
                                 gik = 2.0 * dEd[2] * vik[k];
                    gradient[3 * i + k] += -gij - gik;
                    gradient[3 * j + k] += gij - gjk;
                    gradient[3 * l + k] += gjk + gik;
                }
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b)
                        sigma[3 * a + b] += 2.0 * (dEd[0] * vij[a] * vij[b] + dEd[1] * vjk[a] * vjk[b]
                                                   + dEd[2] * vik[a] * vik[b]);
                /* dE/dc6: c9 = -s9 sqrt(c6ij c6ik c6jk) -> dc9/dc6ij = c9 / (2 c6ij) */
                dEdc6[i * nat + j] += rr * c9 / (2.0 * c6ij);
                dEdc6[i * nat + l] += rr * c9 / (2.0 * c6ik);
                dEdc6[j * nat + l] += rr * c9 / (2.0 * c6jk);
            }
        }
}
