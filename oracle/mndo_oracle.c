/*
 * mndo_oracle.c - test infrastructure: plain-C CPU restatement of pDynamo 1.9.0's NDDO closed-shell RHF
 * energy + analytic gradient path (QCModelMNDO) with Lowdin-charge QC/MM embedding.  It is the checker
 * for the CUDA path and the CPU-baseline port; see mndo_oracle.h.  Dense full matrices are used for
 * clarity; nothing here is tuned.  Paths in citations are relative to the pDynamo project root and
 * "csource/" means pMolecule-1.9.0/extensions/csource/.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "mndo_oracle.h"

/* pCore-1.9.0/extensions/cinclude/Units.h:21,55-58 and pMolecule.MNDOParameters.pyx:18-21. */
#define BOHRS_TO_ANGSTROMS (5.291772083e-11 / 1.0e-10)
#define ANGSTROMS_TO_BOHRS (1.0e-10 / 5.291772083e-11)
#define HARTREES_TO_EV     27.2113834
#define HARTREES_TO_KCAL   (27.2113834 * 23.060529)
/* pMolecule-1.9.0/extensions/cinclude/MNDODefinitions.h:105-111. */
#define EXPONENT_TOLERANCE 25.0
#define PDDG_EXPONENT      (10.0 * BOHRS_TO_ANGSTROMS * BOHRS_TO_ANGSTROMS)
#define SMALL_RIJ          5.0e-3
#define SMALL_RIJ2         2.0e-5
/* csource/MNDOIntegralUtilities.c:449; cinclude/GaussianBasis.h:25,43; csource/QCModelMNDO.c:1029. */
#define ALIGNMENT_TOLERANCE 0.99999999
#define PRIMITIVE_OVERLAP_TOLERANCE (2.30258509299405 * 18.0)
#define TEI_UNDERFLOW 1.0e-12
#define PI 3.14159265358979323846

enum { R_III, R_IIID, R_IR016, R_IR066, R_IR244, R_IR266, R_IR466, R_QND, R_QNP, R_QNS,
       R_AD, R_ALP, R_AM, R_AQ, R_BETAD, R_BETAP, R_BETAS, R_DD, R_EHEAT, R_EISOL, R_F0SD, R_GPHOT,
       R_GPP, R_GP2, R_GSP, R_GSS, R_G2SD, R_HSP, R_PCORE, R_QQ, R_UDD, R_UPP, R_USS, R_ZCORE,
       R_ZETAD, R_ZETAP, R_ZETAS, R_ZDN, R_ZPN, R_ZSN };

typedef struct {
    int Z, norb, iii, nshell, ng, npddg, nprim[2];
    double po[9], ddp[6], dd, qq, am, ad, aq, alp, zcore, eheat, eisol, gss, gsp, gpp, gp2, hsp, hpp, gphot, pcore;
    double beta[4], uspd[4], fn1[4], fn2[4], fn3[4], pddgc[4], pddge[4], zetas, zetap;
    double exps[2][ORACLE_MAXPRIM], ccbf[2][ORACLE_MAXPRIM];
    int ndiat;                                   /* PM6 diatomic core-core pairs, indexed by partner atomic number */
    unsigned char diat_flag[ORACLE_MAXDIATOMIC];
    double diat_a[ORACLE_MAXDIATOMIC], diat_x[ORACLE_MAXDIATOMIC];
} Element;

struct OracleHamiltonian { int n; Element *el; };

static inline int PK(int i, int j) { return (i >= j) ? i * (i + 1) / 2 + j : j * (j + 1) / 2 + i; }

/* ================================================================================================ */
/* Parameters: pMolecule.MNDOParameters.pyx:309-370 (units); csource/MNDOParameters.c:155-240
 * (one-centre TEIs and hpp), :726-735 (AIJL), :762-875 (FillDDPPO), :880-930 (POIJ).               */
static double factorial(int n) { double v = 1.0; for (int i = 1; i <= n; i++) v *= (double)i; return v; }

static double aijl(double z1, double z2, int n1, int n2, int l)
{
    return factorial(n1 + n2 + l) / sqrt(factorial(2 * n1) * factorial(2 * n2)) *
           pow(2.0 * z1 / (z1 + z2), n1) * sqrt(2.0 * z1 / (z1 + z2)) *
           pow(2.0 * z2 / (z1 + z2), n2) * sqrt(2.0 * z2 / (z1 + z2)) * pow(2.0, l) / pow(z1 + z2, l);
}

static double poij(int l, double d, double fg)
{
    if (l == 0) return 0.5 / fg;
    double dsq = d * d, a1 = 0.1, a2 = 5.0, f1 = 0.0, f2 = 0.0;
    for (int i = 0; i < 100; i++) {   /* golden-section search with the reference's constants */
        double delta = a2 - a1;
        if (delta < 1.0e-8) break;
        double y1 = a1 + delta * 0.382, y2 = a1 + delta * 0.618;
        if (l == 1) {
            f1 = pow(0.25 * (1.0 / y1 - 1.0 / sqrt(y1 * y1 + dsq)) - fg, 2);
            f2 = pow(0.25 * (1.0 / y2 - 1.0 / sqrt(y2 * y2 + dsq)) - fg, 2);
        } else {
            f1 = pow(0.125 * (1.0 / y1 - 2.0 / sqrt(y1 * y1 + 0.5 * dsq) + 1.0 / sqrt(y1 * y1 + dsq)) - fg, 2);
            f2 = pow(0.125 * (1.0 / y2 - 2.0 / sqrt(y2 * y2 + 0.5 * dsq) + 1.0 / sqrt(y2 * y2 + dsq)) - fg, 2);
        }
        if (f1 < f2) a2 = y2; else a1 = y1;
    }
    return (f1 >= f2) ? a2 : a1;
}

static void fill_ddp_po(Element *e)
{
    double aij[6] = {0};
    for (int i = 0; i < 6; i++) e->ddp[i] = 0.0;
    for (int i = 0; i < 9; i++) e->po[i] = 0.0;
    if (e->Z > 2 && e->zetas * e->zetap >= 1.0e-2) {
        aij[1] = aijl(e->zetas, e->zetap, e->iii, e->iii, 1);
        aij[2] = aijl(e->zetap, e->zetap, e->iii, e->iii, 2);
    }
    e->po[0] = poij(0, 1.0, e->gss);
    e->po[8] = e->po[0];
    if (e->Z > 2) {
        double d = aij[1] / sqrt(12.0);
        e->ddp[1] = d; e->po[1] = poij(1, d, e->hsp);
        e->po[6] = e->po[0];
        d = sqrt(aij[2] / 10.0);
        e->ddp[2] = d; e->po[2] = poij(2, d, e->hpp);
    }
    /* sp elements: the multipole charge separations and additive terms come from the parameter file. */
    if (e->am < 1.0e-4) e->am = 1.0;
    e->po[0] = 0.5 / e->am;
    if (e->ad > 1.0e-5) e->po[1] = 0.5 / e->ad;
    if (e->aq > 1.0e-5) e->po[2] = 0.5 / e->aq;
    e->po[6] = e->po[0];
    e->po[8] = e->po[0];
    e->ddp[1] = e->dd;
    e->ddp[2] = e->qq * sqrt(2.0);
    if (e->pcore > 1.0e-5) e->po[8] = e->pcore;
}

/* STO-6G shells: GaussianBasis_UnnormalizePrimitives (csource/GaussianBasisCore.c:309), exponent scaling by
 * zeta^2 (:280) and renormalisation of the contracted Cartesian function to unit self-overlap (:221). */
static void make_basis(Element *e, const int *shellTypes, const int *nPrimitives, const double *exps0, const double *coef0)
{
    const double zeta[2] = { e->zetas, e->zetap };
    for (int s = 0; s < e->nshell; s++) {
        int l = shellTypes[s];
        e->nprim[s] = nPrimitives[s];
        for (int p = 0; p < nPrimitives[s]; p++) {
            double ex = 2.0 * exps0[s * ORACLE_MAXPRIM + p];
            double fac = pow(PI, 1.5) / (ex * sqrt(ex));
            if (l == 1) fac *= 1.0 / (2.0 * ex);
            e->ccbf[s][p] = coef0[s * ORACLE_MAXPRIM + p] / sqrt(fac);
            e->exps[s][p] = exps0[s * ORACLE_MAXPRIM + p] * zeta[s] * zeta[s];
        }
        double norm = 0.0;
        for (int p = 0; p < nPrimitives[s]; p++)
            for (int q = 0; q < nPrimitives[s]; q++) {
                double a = e->exps[s][p] + e->exps[s][q];
                double v = pow(PI / a, 1.5);
                if (l == 1) v *= 0.5 / a;
                norm += e->ccbf[s][p] * e->ccbf[s][q] * v;
            }
        for (int p = 0; p < nPrimitives[s]; p++) e->ccbf[s][p] /= sqrt(norm);
    }
}

OracleHamiltonian *oracle_hamiltonian_create(int nElements, const int *atomicNumbers, const int *norbitals,
                                             const double *raw, const int *nGaussians, const double *gaussians,
                                             const int *nPDDG, const double *pddg, const int *nShells,
                                             const int *shellTypes, const int *nPrimitives,
                                             const double *exponents, const double *coefficients,
                                             const int *nDiatomic, const double *diatomic)
{
    OracleHamiltonian *h = (OracleHamiltonian *)calloc(1, sizeof(OracleHamiltonian));
    h->n = nElements;
    h->el = (Element *)calloc(nElements, sizeof(Element));
    for (int k = 0; k < nElements; k++) {
        Element *e = &h->el[k];
        const double *r = raw + k * ORACLE_NRAW;
        e->Z = atomicNumbers[k]; e->norb = norbitals[k]; e->iii = (int)r[R_III];
        if (e->norb != 1 && e->norb != 4) { free(h->el); free(h); return NULL; }
        e->ad = r[R_AD]; e->alp = r[R_ALP] * BOHRS_TO_ANGSTROMS; e->am = r[R_AM]; e->aq = r[R_AQ];
        e->dd = r[R_DD]; e->qq = r[R_QQ]; e->zcore = r[R_ZCORE]; e->gphot = r[R_GPHOT]; e->pcore = r[R_PCORE];
        e->eheat = r[R_EHEAT] / HARTREES_TO_KCAL; e->eisol = r[R_EISOL] / HARTREES_TO_EV;
        e->gss = r[R_GSS] / HARTREES_TO_EV; e->gsp = r[R_GSP] / HARTREES_TO_EV; e->gpp = r[R_GPP] / HARTREES_TO_EV;
        e->gp2 = r[R_GP2] / HARTREES_TO_EV; e->hsp = r[R_HSP] / HARTREES_TO_EV;
        e->hpp = (e->norb >= 4) ? 0.5 * (e->gpp - e->gp2) : 0.0;
        e->zetas = r[R_ZETAS]; e->zetap = r[R_ZETAP];
        e->beta[0] = r[R_BETAS] / HARTREES_TO_EV; e->uspd[0] = r[R_USS] / HARTREES_TO_EV;
        for (int i = 1; i < e->norb; i++) { e->beta[i] = r[R_BETAP] / HARTREES_TO_EV; e->uspd[i] = r[R_UPP] / HARTREES_TO_EV; }
        e->ng = nGaussians[k];
        for (int i = 0; i < e->ng; i++) {
            const double *g = gaussians + (k * ORACLE_MAXGAUSS + i) * 3;
            e->fn1[i] = g[0] / (BOHRS_TO_ANGSTROMS * HARTREES_TO_EV);
            e->fn2[i] = g[1] * BOHRS_TO_ANGSTROMS * BOHRS_TO_ANGSTROMS;
            e->fn3[i] = g[2] / BOHRS_TO_ANGSTROMS;
        }
        e->npddg = nPDDG[k];
        for (int i = 0; i < e->npddg; i++) {
            const double *g = pddg + (k * ORACLE_MAXPDDG + i) * 2;
            e->pddgc[i] = g[0] / HARTREES_TO_EV; e->pddge[i] = g[1] / BOHRS_TO_ANGSTROMS;
        }
        /* PM6 diatomic pairs (pMolecule.MNDOParameters.pyx:259-276, units :358-363: a in bohr^-1 x 0.529..) */
        e->ndiat = 0;
        for (int i = 0; i < nDiatomic[k]; i++) {
            const double *d = diatomic + (k * ORACLE_MAXDIATOMIC + i) * 3;
            int j = (int)d[0];
            if (j < 0 || j >= ORACLE_MAXDIATOMIC) continue;
            e->diat_flag[j] = 1; e->diat_x[j] = d[1]; e->diat_a[j] = d[2] * BOHRS_TO_ANGSTROMS;
            if (j + 1 > e->ndiat) e->ndiat = j + 1;
        }
        fill_ddp_po(e);
        e->nshell = nShells[k];
        make_basis(e, shellTypes + 2 * k, nPrimitives + 2 * k, exponents + k * 2 * ORACLE_MAXPRIM,
                   coefficients + k * 2 * ORACLE_MAXPRIM);
    }
    return h;
}

void oracle_hamiltonian_free(OracleHamiltonian *h) { if (h) { free(h->el); free(h); } }

int oracle_element_derived(const OracleHamiltonian *h, int k, double *out)
{
    if (!h || k < 0 || k >= h->n) return 4;
    const Element *e = &h->el[k];
    int n = 0;
    for (int i = 0; i < 9; i++) out[n++] = e->po[i];
    for (int i = 0; i < 6; i++) out[n++] = e->ddp[i];
    out[n++] = e->dd; out[n++] = e->qq; out[n++] = e->am; out[n++] = e->ad; out[n++] = e->aq; out[n++] = e->alp;
    out[n++] = e->zcore; out[n++] = e->eheat; out[n++] = e->eisol;
    out[n++] = e->gss; out[n++] = e->gsp; out[n++] = e->gpp; out[n++] = e->gp2; out[n++] = e->hsp; out[n++] = e->hpp;
    for (int i = 0; i < 4; i++) out[n++] = (i < e->norb) ? e->beta[i] : 0.0;
    for (int i = 0; i < 4; i++) out[n++] = (i < e->norb) ? e->uspd[i] : 0.0;
    for (int i = 0; i < 4; i++) out[n++] = (i < e->ng) ? e->fn1[i] : 0.0;
    for (int i = 0; i < 4; i++) out[n++] = (i < e->ng) ? e->fn2[i] : 0.0;
    for (int i = 0; i < 4; i++) out[n++] = (i < e->ng) ? e->fn3[i] : 0.0;
    for (int i = 0; i < 4; i++) out[n++] = (i < e->npddg) ? e->pddgc[i] : 0.0;
    for (int i = 0; i < 4; i++) out[n++] = (i < e->npddg) ? e->pddge[i] : 0.0;
    /* one-centre TEI values in the order of MNDOParameters.c:170-215 */
    double oc[16] = { e->gss, e->gpp, e->gpp, e->gpp, e->gsp, e->gsp, e->gsp, e->hsp, e->hsp, e->hsp,
                      e->gp2, e->gp2, e->gp2, e->hpp, e->hpp, e->hpp };
    int noc = (e->norb == 1) ? 1 : 16;
    for (int i = 0; i < 16; i++) out[n++] = (i < noc) ? oc[i] : 0.0;
    for (int i = 0; i < 16; i++) out[n++] = 0.0;
    return 0;
}

/* ================================================================================================ */
/* Core-core repulsion and its r-derivative, non-diatomic branch: csource/MNDOIntegralUtilities.c:35-150
 * (CoreCore) and :152-281 (CoreCoreD).  The diatomic (PM6) branch is outside this path.           */
/* PM6 diatomic core-core term and its r-derivative (csource/MNDOIntegralUtilities.c:45-96 energy, :164-218
 * derivative): scale = 1 + x_ij exp(-a_ij r_A^2)-type pair terms (X-H with X = C, N, O) or
 * x_ij exp(-a_ij r (1 + 0.0003 r_A^5)), the C-C and Si-O extra terms, times Z_a Z_b gamma, plus the
 * unpolarisable core 1e-8 eV A^12 ((Z_a^1/3 + Z_b^1/3) / r_A)^12.                                   */
#define PM6_UNPOLARIZABLE_CORE (1.0e-08 / 27.21)
static double core_core_pm6(const Element *a, const Element *b, double r, double gam, double dgdr, double *scale_rest, double *dedr)
{
    double scale = 1.0, dscale = 0.0, rA = r * BOHRS_TO_ANGSTROMS;
    if (b->Z < a->ndiat && a->diat_flag[b->Z]) {
        double aij = a->diat_a[b->Z], xij = 2.0 * a->diat_x[b->Z];   /* factor 2 as the reference (Stewart's AM1/d) */
        int xh = (a->Z == 1 && (b->Z == 6 || b->Z == 7 || b->Z == 8)) || (b->Z == 1 && (a->Z == 6 || a->Z == 7 || a->Z == 8));
        if (xh) {
            double f3 = xij * exp(-aij * r * r * BOHRS_TO_ANGSTROMS);
            dscale -= 2.0 * aij * r * BOHRS_TO_ANGSTROMS * f3;
            scale += f3;
        } else {
            double dd = 0.0003 * pow(rA, 5), f3 = xij * exp(-aij * r * (1.0 + dd));
            dscale -= aij * (1.0 + 6.0 * dd) * f3;
            scale += f3;
        }
    }
    if (a->Z == 6 && b->Z == 6) {
        double f3 = 9.28 * exp(-5.98 * rA);
        dscale -= 5.98 * BOHRS_TO_ANGSTROMS * f3;
        scale += f3;
    }
    if ((a->Z == 8 && b->Z == 14) || (a->Z == 14 && b->Z == 8)) {
        double dd = rA - 2.9, f3 = -0.0007 * exp(-dd * dd);
        dscale -= 2.0 * dd * BOHRS_TO_ANGSTROMS * f3;
        scale += f3;
    }
    double zz = a->zcore * b->zcore;
    double u = (pow(a->zcore, 1.0 / 3.0) + pow(b->zcore, 1.0 / 3.0)) / rA, u12 = pow(u, 12);
    double enuc = zz * gam * scale + PM6_UNPOLARIZABLE_CORE * u12;
    *dedr = zz * (dgdr * scale + gam * dscale) - 12.0 * PM6_UNPOLARIZABLE_CORE * u12 / r;
    *scale_rest = 0.0;
    return enuc;
}

static double core_core(const Element *a, const Element *b, double r, double *dedr)
{
    double s8 = a->po[8] + b->po[8];
    double gam = 1.0 / sqrt(r * r + s8 * s8), dgdr = -r * gam * gam * gam;
    if (a->ndiat > 0 && b->ndiat > 0) {
        /* PM6: the diatomic term, then the AM1/PM3 Gaussian terms as for the other Hamiltonians */
        double scale, de, enuc = core_core_pm6(a, b, r, gam, dgdr, &scale, &de);
        double zz = a->zcore * b->zcore, an = 0.0;
        const Element *e2[2] = { a, b };
        for (int t = 0; t < 2; t++) {
            const Element *e = e2[t];
            for (int i = 0; i < e->ng; i++) {
                double d = r - e->fn3[i], ax = e->fn2[i] * d * d;
                if (ax <= EXPONENT_TOLERANCE) {
                    scale += a->gphot * b->gphot * zz / r * e->fn1[i] * exp(-ax);
                    an += e->fn1[i] * (1.0 / (r * r) + e->fn2[i] * 2.0 * d / r) * exp(-ax);
                }
            }
        }
        de -= an * a->gphot * b->gphot * zz;
        if (dedr) *dedr = de;
        return enuc + scale;
    }
    double exi = exp(-a->alp * r), exj = exp(-b->alp * r);
    double scale = exi + exj;
    int nt = a->Z + b->Z;
    if (nt == 8 || nt == 9) {
        if (a->Z == 7 || a->Z == 8) scale += (BOHRS_TO_ANGSTROMS * r - 1.0) * exi;
        if (b->Z == 7 || b->Z == 8) scale += (BOHRS_TO_ANGSTROMS * r - 1.0) * exj;
    }
    double zz = a->zcore * b->zcore;
    double enuc = zz * gam;
    scale = fabs(scale * enuc);
    double dd;
    if (a->Z == 1 && (b->Z == 7 || b->Z == 8)) {
        double f3 = 1.0 + exi + BOHRS_TO_ANGSTROMS * r * exj;
        dd = dgdr * f3 - gam * (a->alp * exi + BOHRS_TO_ANGSTROMS * (b->alp * r - 1.0) * exj);
    } else if ((a->Z == 7 || a->Z == 8) && b->Z == 1) {
        double f3 = 1.0 + exj + BOHRS_TO_ANGSTROMS * r * exi;
        dd = dgdr * f3 - gam * (b->alp * exj + BOHRS_TO_ANGSTROMS * (a->alp * r - 1.0) * exi);
    } else {
        double f3 = 1.0 + exi + exj;
        dd = dgdr * f3 - gam * (a->alp * exi + b->alp * exj);
    }
    double de = zz * dd;
    double an = 0.0;
    const Element *e2[2] = { a, b };
    for (int t = 0; t < 2; t++) {
        const Element *e = e2[t];
        for (int i = 0; i < e->ng; i++) {
            double d = r - e->fn3[i], ax = e->fn2[i] * d * d;
            if (ax <= EXPONENT_TOLERANCE) {
                scale += a->gphot * b->gphot * zz / r * e->fn1[i] * exp(-ax);
                an += e->fn1[i] * (1.0 / (r * r) + e->fn2[i] * 2.0 * d / r) * exp(-ax);
            }
        }
    }
    de -= an * a->gphot * b->gphot * zz;
    if (a->npddg > 0 && b->npddg > 0) {
        double zaf = a->zcore / (a->zcore + b->zcore), zbf = b->zcore / (a->zcore + b->zcore), ap = 0.0;
        for (int i = 0; i < a->npddg; i++)
            for (int j = 0; j < b->npddg; j++) {
                double d = r - a->pddge[i] - b->pddge[j], ax = PDDG_EXPONENT * d * d;
                double c = zaf * a->pddgc[i] + zbf * b->pddgc[j];
                scale += c * exp(-ax);
                ap += c * 2.0 * PDDG_EXPONENT * d * exp(-ax);
            }
        de -= ap;
    }
    if (dedr) *dedr = de;
    return enuc + scale;
}

/* ================================================================================================ */
/* Local-frame two-centre integrals of the sp multipole model (REPP equivalent) and their r-derivatives:
 * csource/MNDOIntegralUtilities.c:1117-1171 (electron-core) and :1180-1440 (TEIs), symmetry copies
 * :909-1100 with the SPPOSITIVE/SPOSITIVE/CPOSITIVE tables of cinclude/MNDOIntegralDefinitions.h.
 * Local orbitals: 0 s, 1 p-sigma, 2 p-pi+, 3 p-pi-; distributions packed i(i+1)/2+j.               */
enum { SS = 0, PZS = 1, PZPZ = 2, PXS = 3, PXPZ = 4, PXPX = 5, PYS = 6, PYPZ = 7, PYPX = 8, PYPY = 9 };

static void local_core(const Element *a, const Element *b, double r, int swapped, double *c, double *dc)
{
    /* electron distribution on a, core of b */
    for (int i = 0; i < 10; i++) { c[i] = 0.0; dc[i] = 0.0; }
    double rsq = r * r, t = a->po[0] + b->po[8];
    double ri0 = 1.0 / sqrt(rsq + t * t);
    c[SS] = ri0; dc[SS] = -r * ri0 * ri0 * ri0;
    if (a->norb > 3) {
        double da = a->dd, qa = a->qq * 2.0;
        if (swapped) { da = -da; qa = -qa; }
        double aee = pow(a->po[6] + b->po[8], 2), ade = pow(a->po[1] + b->po[8], 2), aqe = pow(a->po[2] + b->po[8], 2);
        double x, s1, s2, s3, s4, s5, s6;
        x = r + da; s1 = 1.0 / sqrt(x * x + ade);
        x = r - da; s2 = 1.0 / sqrt(x * x + ade);
        x = r + qa; s3 = 1.0 / sqrt(x * x + aqe);
        x = r - qa; s4 = 1.0 / sqrt(x * x + aqe);
        x = rsq + aqe; s5 = 1.0 / sqrt(x); s6 = 1.0 / sqrt(x + qa * qa);
        double dze = -0.5 * (s1 - s2), qzze = 0.25 * (s3 + s4) - 0.5 * s5, qxxe = 0.5 * (s6 - s5);
        ri0 = 1.0 / sqrt(rsq + aee);
        c[PZS] = dze; c[PZPZ] = ri0 + qzze; c[PXPX] = ri0 + qxxe;
        double xx = r * s5 * s5 * s5;
        double gdze = 0.5 * ((r + da) * s1 * s1 * s1 - (r - da) * s2 * s2 * s2);
        double gqzze = -0.25 * ((r + qa) * s3 * s3 * s3 + (r - qa) * s4 * s4 * s4) + 0.5 * xx;
        double gqxxe = -0.5 * (r * s6 * s6 * s6 - xx);
        double gri0 = -r * ri0 * ri0 * ri0;
        dc[PZS] = gdze; dc[PZPZ] = gri0 + gqzze; dc[PXPX] = gri0 + gqxxe;
        c[PYPY] = c[PXPX]; dc[PYPY] = dc[PXPX];
    }
    for (int i = 0; i < 10; i++) { c[i] *= -b->zcore; dc[i] *= -b->zcore; }
}

static void local_teis(const Element *a, const Element *b, double r, double L[10][10], double D[10][10])
{
    for (int i = 0; i < 10; i++) for (int j = 0; j < 10; j++) { L[i][j] = 0.0; D[i][j] = 0.0; }
    double rsq = r * r, t = a->po[0] + b->po[0];
    double ri0 = 1.0 / sqrt(rsq + t * t), gri0 = -r * ri0 * ri0 * ri0;
    L[SS][SS] = ri0; D[SS][SS] = gri0;
    double da = 0, qa = 0, db = 0, qb = 0, dze = 0, qzze = 0, qxxe = 0, edz = 0, eqzz = 0, eqxx = 0;
    double gdze = 0, gqzze = 0, gqxxe = 0, gedz = 0, geqzz = 0, geqxx = 0;
    if (a->norb > 3) {
        da = a->dd; qa = a->qq * 2.0;
        double ade = pow(a->po[1] + b->po[0], 2), aqe = pow(a->po[2] + b->po[0], 2), x, s1, s2, s3, s4, s5, s6;
        x = r + da; s1 = 1.0 / sqrt(x * x + ade);
        x = r - da; s2 = 1.0 / sqrt(x * x + ade);
        x = r + qa; s3 = 1.0 / sqrt(x * x + aqe);
        x = r - qa; s4 = 1.0 / sqrt(x * x + aqe);
        x = rsq + aqe; s5 = 1.0 / sqrt(x); s6 = 1.0 / sqrt(x + qa * qa);
        dze = -0.5 * (s1 - s2); qzze = 0.25 * (s3 + s4) - 0.5 * s5; qxxe = 0.5 * (s6 - s5);
        L[PZS][SS] = dze; L[PZPZ][SS] = ri0 + qzze; L[PXPX][SS] = ri0 + qxxe;
        double xx = r * s5 * s5 * s5;
        gdze = 0.5 * ((r + da) * s1 * s1 * s1 - (r - da) * s2 * s2 * s2);
        gqzze = -0.25 * ((r + qa) * s3 * s3 * s3 + (r - qa) * s4 * s4 * s4) + 0.5 * xx;
        gqxxe = -0.5 * (r * s6 * s6 * s6 - xx);
        D[PZS][SS] = gdze; D[PZPZ][SS] = gri0 + gqzze; D[PXPX][SS] = gri0 + gqxxe;
    }
    if (b->norb > 3) {
        db = b->dd; qb = b->qq * 2.0;
        double aed = pow(a->po[0] + b->po[1], 2), aeq = pow(a->po[0] + b->po[2], 2), x, s7, s8, s9, s10, s11, s12;
        x = r - db; s7 = 1.0 / sqrt(x * x + aed);
        x = r + db; s8 = 1.0 / sqrt(x * x + aed);
        x = r - qb; s9 = 1.0 / sqrt(x * x + aeq);
        x = r + qb; s10 = 1.0 / sqrt(x * x + aeq);
        x = rsq + aeq; s11 = 1.0 / sqrt(x); s12 = 1.0 / sqrt(x + qb * qb);
        edz = -0.5 * (s7 - s8); eqzz = 0.25 * (s9 + s10) - 0.5 * s11; eqxx = 0.5 * (s12 - s11);
        L[SS][PZS] = edz; L[SS][PZPZ] = ri0 + eqzz; L[SS][PXPX] = ri0 + eqxx;
        double xx = r * s11 * s11 * s11;
        gedz = 0.5 * ((r - db) * s7 * s7 * s7 - (r + db) * s8 * s8 * s8);
        geqzz = -0.25 * ((r - qb) * s9 * s9 * s9 + (r + qb) * s10 * s10 * s10) + 0.5 * xx;
        geqxx = -0.5 * (r * s12 * s12 * s12 - xx);
        D[SS][PZS] = gedz; D[SS][PZPZ] = gri0 + geqzz; D[SS][PXPX] = gri0 + geqxx;
    }
    if (a->norb > 3 && b->norb > 3) {
        double axx = pow(a->po[1] + b->po[1], 2), adq = pow(a->po[1] + b->po[2], 2);
        double aqd = pow(a->po[2] + b->po[1], 2), aqq = pow(a->po[2] + b->po[2], 2);
        double s[72], x, y, z, w;
#define RS(k, v) s[k] = 1.0 / sqrt(v)
        x = da - db; RS(13, rsq + axx + x * x);
        x = da + db; RS(14, rsq + axx + x * x);
        x = r + da - db; RS(15, x * x + axx);
        x = r - da + db; RS(16, x * x + axx);
        x = r - da - db; RS(17, x * x + axx);
        x = r + da + db; RS(18, x * x + axx);
        x = r + da; y = x * x + adq; RS(19, y); RS(20, y + qb * qb);
        x = r - da; y = x * x + adq; RS(21, y); RS(22, y + qb * qb);
        x = r - db; y = x * x + aqd; RS(23, y); RS(24, y + qa * qa);
        x = r + db; y = x * x + aqd; RS(25, y); RS(26, y + qa * qa);
        x = r + da - qb; RS(27, x * x + adq);
        x = r - da - qb; RS(28, x * x + adq);
        x = r + da + qb; RS(29, x * x + adq);
        x = r - da + qb; RS(30, x * x + adq);
        x = r + qa - db; RS(31, x * x + aqd);
        x = r + qa + db; RS(32, x * x + aqd);
        x = r - qa - db; RS(33, x * x + aqd);
        x = r - qa + db; RS(34, x * x + aqd);
        double a35 = rsq + aqq; RS(35, a35);
        x = qa - qb; RS(36, a35 + x * x);
        x = qa + qb; RS(37, a35 + x * x);
        x = a35 + qa * qa; RS(38, x); RS(39, a35 + qb * qb); RS(40, x + qb * qb);
        x = r - qb; y = x * x + aqq; RS(41, y); RS(42, y + qa * qa);
        x = r + qb; y = x * x + aqq; RS(43, y); RS(44, y + qa * qa);
        x = r + qa; y = x * x + aqq; RS(45, y); RS(46, y + qb * qb);
        x = r - qa; y = x * x + aqq; RS(47, y); RS(48, y + qb * qb);
        x = r + qa - qb; RS(49, x * x + aqq);
        x = r + qa + qb; RS(50, x * x + aqq);
        x = r - qa - qb; RS(51, x * x + aqq);
        x = r - qa + qb; RS(52, x * x + aqq);
        double qa0 = a->qq, qb0 = b->qq;
        x = pow(da - qb0, 2); y = pow(r - qb0, 2); z = pow(da + qb0, 2); w = pow(r + qb0, 2);
        RS(53, x + y + adq); RS(54, x + w + adq); RS(55, z + y + adq); RS(56, z + w + adq);
        x = pow(qa0 - db, 2); y = pow(qa0 + db, 2); z = pow(r + qa0, 2); w = pow(r - qa0, 2);
        RS(57, z + x + aqd); RS(58, w + x + aqd); RS(59, z + y + aqd); RS(60, w + y + aqd);
        x = pow(qa0 - qb0, 2); y = pow(qa0 + qb0, 2);
        z = pow(r + qa0 - qb0, 2); RS(64, z + x + aqq); RS(65, z + y + aqq);
        z = pow(r + qa0 + qb0, 2); RS(66, z + x + aqq); RS(67, z + y + aqq);
        z = pow(r - qa0 - qb0, 2); RS(68, z + x + aqq); RS(69, z + y + aqq);
        z = pow(r - qa0 + qb0, 2); RS(70, z + x + aqq); RS(71, z + y + aqq);
#undef RS
        const double E1 = 0.5, E2 = 0.25, E3 = 0.125, E4 = 0.0625;
        double dxdx = E1 * s[13] - E1 * s[14];
        double dzdz = E2 * s[15] + E2 * s[16] - E2 * s[17] - E2 * s[18];
        double dzqxx = E2 * s[19] - E2 * s[20] - E2 * s[21] + E2 * s[22];
        double qxxdz = E2 * s[23] - E2 * s[24] - E2 * s[25] + E2 * s[26];
        double dzqzz = -E3 * s[27] + E3 * s[28] - E3 * s[29] + E3 * s[30] - E2 * s[21] + E2 * s[19];
        double qzzdz = -E3 * s[31] + E3 * s[32] - E3 * s[33] + E3 * s[34] + E2 * s[23] - E2 * s[25];
        double qxxqxx = E3 * s[36] + E3 * s[37] - E2 * s[38] - E2 * s[39] + E2 * s[35];
        double qxxqyy = E2 * s[40] - E2 * s[38] - E2 * s[39] + E2 * s[35];
        double qxxqzz = E3 * s[42] + E3 * s[44] - E3 * s[41] - E3 * s[43] - E2 * s[38] + E2 * s[35];
        double qzzqxx = E3 * s[46] + E3 * s[48] - E3 * s[45] - E3 * s[47] - E2 * s[39] + E2 * s[35];
        double qzzqzz = E4 * s[49] + E4 * s[50] + E4 * s[51] + E4 * s[52] - E3 * s[47] - E3 * s[45] - E3 * s[41] - E3 * s[43] + E2 * s[35];
        double dxqxz = -E2 * s[53] + E2 * s[54] + E2 * s[55] - E2 * s[56];
        double qxzdx = -E2 * s[57] + E2 * s[58] + E2 * s[59] - E2 * s[60];
        double qxzqxz = E3 * s[64] - E3 * s[66] - E3 * s[68] + E3 * s[70] - E3 * s[65] + E3 * s[67] + E3 * s[69] - E3 * s[71];
        L[PZS][PZS] = dzdz; L[PXS][PXS] = dxdx;
        L[PZPZ][PZS] = edz + qzzdz; L[PXPX][PZS] = edz + qxxdz; L[PXPZ][PXS] = qxzdx;
        L[PZS][PZPZ] = dze + dzqzz; L[PZS][PXPX] = dze + dzqxx; L[PXS][PXPZ] = dxqxz;
        L[PZPZ][PZPZ] = ri0 + eqzz + qzze + qzzqzz; L[PXPX][PZPZ] = ri0 + eqzz + qxxe + qxxqzz;
        L[PZPZ][PXPX] = ri0 + eqxx + qzze + qzzqxx; L[PXPX][PXPX] = ri0 + eqxx + qxxe + qxxqxx;
        L[PXPZ][PXPZ] = qxzqxz; L[PXPX][PYPY] = ri0 + eqxx + qxxe + qxxqyy; L[PYPX][PYPX] = 0.5 * (qxxqxx - qxxqyy);
        /* derivatives */
#define C3(k) (s[k] * s[k] * s[k])
        double g13 = -E1 * r * (C3(13) - C3(14));
        double gzz = -E2 * ((r + da - db) * C3(15) + (r - da + db) * C3(16) - (r - da - db) * C3(17) - (r + da + db) * C3(18));
        double ww = (r + da) * C3(19), xx = (r - da) * C3(21);
        double gdzqxx = -E2 * (ww - (r + da) * C3(20) - xx + (r - da) * C3(22));
        double yy = (r - db) * C3(23), zz = (r + db) * C3(25);
        double gqxxdz = -E2 * (yy - (r - db) * C3(24) - zz + (r + db) * C3(26));
        double gdzqzz = -E3 * (-(r + da - qb) * C3(27) + (r - da - qb) * C3(28) - (r + da + qb) * C3(29) + (r - da + qb) * C3(30)) + E2 * (xx - ww);
        double gqzzdz = -E3 * (-(r + qa - db) * C3(31) + (r + qa + db) * C3(32) - (r - qa - db) * C3(33) + (r - qa + db) * C3(34)) - E2 * (yy - zz);
        double g35 = r * C3(35), g38 = r * C3(38), g39 = r * C3(39);
        double gqxxqxx = -E3 * (r * C3(36) + r * C3(37)) + E2 * (g38 + g39 - g35);
        double gqxxqyy = -E2 * (r * C3(40) - g38 - g39 + g35);
        ww = (r - qb) * C3(41); xx = (r + qb) * C3(43); yy = (r + qa) * C3(45); zz = (r - qa) * C3(47);
        double gqxxqzz = -E3 * ((r - qb) * C3(42) + (r + qb) * C3(44) - ww - xx) + E2 * (g38 - g35);
        double gqzzqxx = -E3 * ((r + qa) * C3(46) + (r - qa) * C3(48) - yy - zz) + E2 * (g39 - g35);
        double gqzzqzz = -E4 * ((r + qa - qb) * C3(49) + (r + qa + qb) * C3(50) + (r - qa - qb) * C3(51) + (r - qa + qb) * C3(52)) + E3 * (zz + yy + ww + xx) - E2 * g35;
        double gdxqxz = -E2 * (-(r - qb0) * C3(53) + (r + qb0) * C3(54) + (r - qb0) * C3(55) - (r + qb0) * C3(56));
        double gqxzdx = -E2 * (-(r + qa0) * C3(57) + (r - qa0) * C3(58) + (r + qa0) * C3(59) - (r - qa0) * C3(60));
        double gqxzqxz = -E3 * ((r + qa0 - qb0) * C3(64) - (r + qa0 + qb0) * C3(66) - (r - qa0 - qb0) * C3(68) + (r - qa0 + qb0) * C3(70) -
                                (r + qa0 - qb0) * C3(65) + (r + qa0 + qb0) * C3(67) + (r - qa0 - qb0) * C3(69) - (r - qa0 + qb0) * C3(71));
#undef C3
        D[PZS][PZS] = gzz; D[PXS][PXS] = g13;
        D[PZPZ][PZS] = gedz + gqzzdz; D[PXPX][PZS] = gedz + gqxxdz; D[PXPZ][PXS] = gqxzdx;
        D[PZS][PZPZ] = gdze + gdzqzz; D[PZS][PXPX] = gdze + gdzqxx; D[PXS][PXPZ] = gdxqxz;
        D[PZPZ][PZPZ] = gri0 + geqzz + gqzze + gqzzqzz; D[PXPX][PZPZ] = gri0 + geqzz + gqxxe + gqxxqzz;
        D[PZPZ][PXPX] = gri0 + geqxx + gqzze + gqzzqxx; D[PXPX][PXPX] = gri0 + geqxx + gqxxe + gqxxqxx;
        D[PXPZ][PXPZ] = gqxzqxz; D[PXPX][PYPY] = gri0 + geqxx + gqxxe + gqxxqyy; D[PYPX][PYPX] = 0.5 * (gqxxqxx - gqxxqyy);
    }
    /* symmetry-related integrals (SPPOSITIVE, SPOSITIVE) */
    double (*M[2])[10] = { L, D };
    for (int t = 0; t < 2; t++) {
        double (*X)[10] = M[t];
        if (b->norb > 3) X[SS][PYPY] = X[SS][PXPX];
        if (a->norb > 3) X[PYPY][SS] = X[PXPX][SS];
        if (a->norb > 3 && b->norb > 3) {
            X[PZS][PYPY] = X[PZS][PXPX]; X[PZPZ][PYPY] = X[PZPZ][PXPX]; X[PYS][PYS] = X[PXS][PXS];
            X[PYS][PYPZ] = X[PXS][PXPZ]; X[PYPZ][PYS] = X[PXPZ][PXS]; X[PYPZ][PYPZ] = X[PXPZ][PXPZ];
            X[PYPY][PZS] = X[PXPX][PZS]; X[PYPY][PZPZ] = X[PXPX][PZPZ]; X[PYPY][PXPX] = X[PXPX][PYPY];
            X[PYPY][PYPY] = X[PXPX][PXPX];
        }
    }
}

/* ================================================================================================ */
/* Rotation from the local to the molecular frame and its Cartesian derivatives (with respect to the
 * coordinates of atom j): csource/MNDOIntegralUtilities.c:449-903 for s/p.  Molecular orbital order
 * s, pz, px, py.  C[ij][mn] is the pair-distribution transform.  Returns r (Bohr).                 */
static double rotation(const double *xi, const double *xj, int norb, double C[10][10], double CD[3][10][10], double v[3])
{
    double x = xj[0] - xi[0], y = xj[1] - xi[1], z = xj[2] - xi[2];
    double r2 = x * x + y * y + z * z, r = sqrt(r2);
    v[0] = x; v[1] = y; v[2] = z;
    for (int i = 0; i < 10; i++) for (int j = 0; j < 10; j++) { C[i][j] = (i == j) ? 1.0 : 0.0; CD[0][i][j] = CD[1][i][j] = CD[2][i][j] = 0.0; }
    if (norb <= 1 || r2 <= SMALL_RIJ2) return r;
    double T[4][4] = {{0}}, TD[3][4][4] = {{{0}}};
    int swapped = fabs(z / r) > ALIGNMENT_TOLERANCE;
    if (swapped) { double t = x; x = z; z = t; }
    double b2 = x * x + y * y, b = sqrt(b2), sb = b / r, ca = x / b, sa = y / b, cb = z / r;
    const int S_ = 0, PZ_ = 1, PX_ = 2, PY_ = 3;
    T[S_][0] = 1.0;
    T[PX_][1] = ca * sb; T[PX_][2] = ca * cb; T[PX_][3] = -sa;
    T[PY_][1] = sa * sb; T[PY_][2] = sa * cb; T[PY_][3] = ca;
    T[PZ_][1] = cb;      T[PZ_][2] = -sb;
    double caX = y * y / (b2 * b), caY = -x * y / (b2 * b), saX = caY, saY = x * x / (b2 * b);
    double cbX = -x * z / (r2 * r), cbY = -y * z / (r2 * r), cbZ = b2 / (r2 * r);
    double sbX = x * z * z / (b * r2 * r), sbY = y * z * z / (b * r2 * r), sbZ = -b * z / (r2 * r);
    TD[0][PX_][1] = caX * sb + ca * sbX; TD[0][PX_][2] = caX * cb + ca * cbX; TD[0][PX_][3] = -saX;
    TD[0][PY_][1] = saX * sb + sa * sbX; TD[0][PY_][2] = saX * cb + sa * cbX; TD[0][PY_][3] = caX;
    TD[0][PZ_][1] = cbX; TD[0][PZ_][2] = -sbX;
    TD[1][PX_][1] = caY * sb + ca * sbY; TD[1][PX_][2] = caY * cb + ca * cbY; TD[1][PX_][3] = -saY;
    TD[1][PY_][1] = saY * sb + sa * sbY; TD[1][PY_][2] = saY * cb + sa * cbY; TD[1][PY_][3] = caY;
    TD[1][PZ_][1] = cbY; TD[1][PZ_][2] = -sbY;
    TD[2][PX_][1] = ca * sbZ; TD[2][PX_][2] = ca * cbZ;
    TD[2][PY_][1] = sa * sbZ; TD[2][PY_][2] = sa * cbZ;
    TD[2][PZ_][1] = cbZ; TD[2][PZ_][2] = -sbZ;
    if (swapped) {   /* premultiply by the x<->z swap and exchange the x and z derivative matrices */
        for (int c = 0; c < 4; c++) {
            double t = T[PX_][c]; T[PX_][c] = T[PZ_][c]; T[PZ_][c] = t;
            for (int k = 0; k < 3; k++) { t = TD[k][PX_][c]; TD[k][PX_][c] = TD[k][PZ_][c]; TD[k][PZ_][c] = t; }
        }
        for (int i = 0; i < 4; i++) for (int c = 0; c < 4; c++) { double t = TD[0][i][c]; TD[0][i][c] = TD[2][i][c]; TD[2][i][c] = t; }
    }
    int ij = 0;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j <= i; j++, ij++) {
            int mn = 0;
            for (int m = 0; m < 4; m++) {
                for (int n = 0; n < m; n++, mn++) {
                    C[ij][mn] = T[i][m] * T[j][n] + T[i][n] * T[j][m];
                    for (int k = 0; k < 3; k++)
                        CD[k][ij][mn] = TD[k][i][m] * T[j][n] + T[i][m] * TD[k][j][n] + TD[k][i][n] * T[j][m] + T[i][n] * TD[k][j][m];
                }
                C[ij][mn] = T[i][m] * T[j][m];
                for (int k = 0; k < 3; k++) CD[k][ij][mn] = TD[k][i][m] * T[j][m] + T[i][m] * TD[k][j][m];
                mn++;
            }
        }
    return r;
}

/* ================================================================================================ */
/* STO-6G overlap between the orbital shells of two atoms and its derivative with respect to the first
 * atom's coordinates (GaussianBasis_2Overlap / _2OverlapD, csource/GaussianBasisCore.c:469,570), mapped
 * to orbital order s, pz, px, py (the spherical p order z, x, y of QCModelMNDO_TransformIntegrals,
 * csource/QCModelMNDO.c:1871).                                                                     */
static void overlap(const Element *ea, const double *A, const Element *eb, const double *B, double S[4][4], double SD[3][4][4])
{
    static const int ORB[3] = { 2, 3, 1 };   /* Cartesian x, y, z -> orbital index */
    double AB[3] = { B[0] - A[0], B[1] - A[1], B[2] - A[2] };
    double R2 = AB[0] * AB[0] + AB[1] * AB[1] + AB[2] * AB[2];
    for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) { S[i][j] = 0.0; SD[0][i][j] = SD[1][i][j] = SD[2][i][j] = 0.0; }
    for (int sa = 0; sa < ea->nshell; sa++)
        for (int sb = 0; sb < eb->nshell; sb++)
            for (int p = 0; p < ea->nprim[sa]; p++)
                for (int q = 0; q < eb->nprim[sb]; q++) {
                    double a = ea->exps[sa][p], b = eb->exps[sb][q], g = a + b;
                    double fac = a * b * R2 / g;
                    if (fac > PRIMITIVE_OVERLAP_TOLERANCE) continue;
                    double s0 = ea->ccbf[sa][p] * eb->ccbf[sb][q] * pow(PI / g, 1.5) * exp(-fac);
                    double PA[3], PB[3], h = 0.5 / g;
                    for (int k = 0; k < 3; k++) { PA[k] = b / g * AB[k]; PB[k] = -a / g * AB[k]; }
                    if (sa == 0 && sb == 0) {
                        S[0][0] += s0;
                        for (int k = 0; k < 3; k++) SD[k][0][0] += 2.0 * a * PA[k] * s0;
                    } else if (sa == 1 && sb == 0) {
                        for (int i = 0; i < 3; i++) {
                            S[ORB[i]][0] += PA[i] * s0;
                            for (int k = 0; k < 3; k++)
                                SD[k][ORB[i]][0] += (2.0 * a * (PA[i] * PA[k] + (i == k) * h) - (i == k)) * s0;
                        }
                    } else if (sa == 0 && sb == 1) {
                        for (int j = 0; j < 3; j++) {
                            S[0][ORB[j]] += PB[j] * s0;
                            for (int k = 0; k < 3; k++) SD[k][0][ORB[j]] += 2.0 * a * (PA[k] * PB[j] + (k == j) * h) * s0;
                        }
                    } else {
                        for (int i = 0; i < 3; i++)
                            for (int j = 0; j < 3; j++) {
                                S[ORB[i]][ORB[j]] += (PA[i] * PB[j] + (i == j) * h) * s0;
                                for (int k = 0; k < 3; k++) {
                                    double dpp = PA[i] * PA[k] * PB[j] + ((i == k) * PB[j] + (i == j) * PA[k] + (k == j) * PA[i]) * h;
                                    SD[k][ORB[i]][ORB[j]] += (2.0 * a * dpp - (i == k) * PB[j]) * s0;
                                }
                            }
                    }
                }
}

/* ================================================================================================ */
/* Integrals of a configuration: csource/QCModelMNDO.c:1032-1160 (QCModelMNDO_Integrals) with
 * csource/MNDOIntegrals.c:147-272 (MolecularFrame2CIntegrals).  Two-centre TEI blocks are kept per
 * atom pair in molecular-frame distribution order (ij on atom i, kl on atom j, i > j).             */
typedef struct {
    int nAtoms, nBasis, *start, *norb;
    const Element **el;
    double *xyz;          /* Bohr */
    double *H;            /* full N x N */
    double *tei;          /* per pair i>j: 100 doubles */
    double enuc;
} Config;

static void config_init(Config *c, const OracleHamiltonian *h, int nAtoms, const int *elementIndex, const double *xyz)
{
    c->nAtoms = nAtoms;
    c->start = (int *)malloc(sizeof(int) * nAtoms);
    c->norb = (int *)malloc(sizeof(int) * nAtoms);
    c->el = (const Element **)malloc(sizeof(Element *) * nAtoms);
    c->xyz = (double *)malloc(sizeof(double) * 3 * nAtoms);
    int n = 0;
    for (int i = 0; i < nAtoms; i++) {
        c->el[i] = &h->el[elementIndex[i]];
        c->start[i] = n; c->norb[i] = c->el[i]->norb; n += c->norb[i];
        for (int k = 0; k < 3; k++) c->xyz[3 * i + k] = xyz[3 * i + k] * ANGSTROMS_TO_BOHRS;
    }
    c->nBasis = n;
    c->H = (double *)calloc((size_t)n * n, sizeof(double));
    c->tei = (double *)calloc((size_t)nAtoms * (nAtoms - 1) / 2 * 100 + 1, sizeof(double));
    c->enuc = 0.0;
}

static void config_free(Config *c) { free(c->start); free(c->norb); free(c->el); free(c->xyz); free(c->H); free(c->tei); }

static inline int pair_index(int i, int j) { return i * (i - 1) / 2 + j; }   /* i > j */

static void integrals(Config *c)
{
    int N = c->nBasis;
    for (int i = 0; i < c->nAtoms; i++) {
        const Element *ei = c->el[i];
        int is = c->start[i];
        for (int m = 0; m < ei->norb; m++) c->H[(is + m) * N + is + m] += ei->uspd[m];
        for (int j = 0; j < i; j++) {
            const Element *ej = c->el[j];
            int js = c->start[j];
            double S[4][4], SD[3][4][4];
            overlap(ei, c->xyz + 3 * i, ej, c->xyz + 3 * j, S, SD);
            for (int m = 0; m < ei->norb; m++)
                for (int n = 0; n < ej->norb; n++) {
                    double v = S[m][n] * 0.5 * (ei->beta[m] + ej->beta[n]);
                    c->H[(is + m) * N + js + n] += v; c->H[(js + n) * N + is + m] += v;
                }
            double Ci[10][10], Cj[10][10], CD[3][10][10], v3[3], L[10][10], LD[10][10], c1[10], d1[10], c2[10], d2[10];
            double r = rotation(c->xyz + 3 * i, c->xyz + 3 * j, ei->norb > ej->norb ? ei->norb : ej->norb, Ci, CD, v3);
            memcpy(Cj, Ci, sizeof(Ci));
            local_teis(ei, ej, r, L, LD);
            local_core(ei, ej, r, 0, c1, d1);
            local_core(ej, ei, r, 1, c2, d2);
            int ni = ei->norb * (ei->norb + 1) / 2, nj = ej->norb * (ej->norb + 1) / 2;
            double *blk = c->tei + (size_t)pair_index(i, j) * 100;
            for (int a = 0; a < ni; a++)
                for (int b = 0; b < nj; b++) {
                    double v = 0.0;
                    for (int p = 0; p < ni; p++)
                        for (int q = 0; q < nj; q++) v += Ci[a][p] * L[p][q] * Cj[b][q];
                    blk[a * 10 + b] = v;
                }
            /* electron-core attraction added to the diagonal blocks */
            int ab = 0;
            for (int a = 0; a < ei->norb; a++)
                for (int b = 0; b <= a; b++, ab++) {
                    double v = 0.0;
                    for (int p = 0; p < ni; p++) v += Ci[ab][p] * c1[p];
                    c->H[(is + a) * N + is + b] += v; if (a != b) c->H[(is + b) * N + is + a] += v;
                }
            ab = 0;
            for (int a = 0; a < ej->norb; a++)
                for (int b = 0; b <= a; b++, ab++) {
                    double v = 0.0;
                    for (int p = 0; p < nj; p++) v += Cj[ab][p] * c2[p];
                    c->H[(js + a) * N + js + b] += v; if (a != b) c->H[(js + b) * N + js + a] += v;
                }
            c->enuc += core_core(ei, ej, r, NULL);
        }
    }
}

/* Two-electron part G(P) of the Fock matrix from the one-centre TEIs (csource/MNDOParameters.c:170-215)
 * and the stored two-centre blocks: G_mn = sum_ls P_ls [(mn|ls) - (ml|ns)/2]
 * (csource/MNDOIntegrals.c:51-143 on the same integral list; values with |v| <= 1e-12 are dropped as
 * cinclude BlockStorage does).                                                                    */
static void fock_g(const Config *c, const double *P, double *G)
{
    int N = c->nBasis;
    memset(G, 0, sizeof(double) * N * N);
    for (int i = 0; i < c->nAtoms; i++) {
        const Element *e = c->el[i];
        int s = c->start[i];
        if (fabs(e->gss) > TEI_UNDERFLOW) G[s * N + s] += 0.5 * P[s * N + s] * e->gss;
        if (e->norb == 4) {
            for (int p = 1; p < 4; p++) {
                int pp = s + p;
                G[s * N + s] += P[pp * N + pp] * (e->gsp - 0.5 * e->hsp);
                G[pp * N + pp] += P[s * N + s] * (e->gsp - 0.5 * e->hsp) + 0.5 * P[pp * N + pp] * e->gpp;
                double v = P[s * N + pp] * (1.5 * e->hsp - 0.5 * e->gsp);
                G[s * N + pp] += v; G[pp * N + s] += v;
                for (int q = 1; q < 4; q++) {
                    if (q == p) continue;
                    int qq = s + q;
                    G[pp * N + pp] += P[qq * N + qq] * (e->gp2 - 0.5 * e->hpp);
                    G[pp * N + qq] += P[pp * N + qq] * (1.5 * e->hpp - 0.5 * e->gp2);
                }
            }
        }
        for (int j = 0; j < i; j++) {
            const double *blk = c->tei + (size_t)pair_index(i, j) * 100;
            int is = c->start[i], js = c->start[j], ni = c->norb[i], nj = c->norb[j];
            int ab = 0;
            for (int a = 0; a < ni; a++)
                for (int b = 0; b <= a; b++, ab++) {
                    int cd = 0;
                    for (int cc = 0; cc < nj; cc++)
                        for (int d = 0; d <= cc; d++, cd++) {
                            double v = blk[ab * 10 + cd];
                            if (fabs(v) <= TEI_UNDERFLOW) continue;
                            /* all orderings (ab|cd), (ba|cd), (ab|dc), (ba|dc) */
                            int A[2] = { is + a, is + b }, B[2] = { js + cc, js + d };
                            int na = (a == b) ? 1 : 2, nb = (cc == d) ? 1 : 2;
                            for (int u = 0; u < na; u++)
                                for (int w = 0; w < nb; w++) {
                                    int m = A[u], n = A[1 - u], l = B[w], sg = B[1 - w];
                                    if (na == 1) n = m;
                                    if (nb == 1) sg = l;
                                    G[m * N + n] += v * P[l * N + sg];          /* Coulomb on the i block */
                                    G[l * N + sg] += v * P[m * N + n];          /* Coulomb on the j block */
                                    G[m * N + l] -= 0.5 * v * P[n * N + sg];    /* exchange, i-j block */
                                    G[l * N + m] -= 0.5 * v * P[n * N + sg];
                                }
                        }
                }
        }
    }
}

/* ================================================================================================ */
/* Symmetric eigensolver (Householder tridiagonalisation + implicit QL with Wilkinson shifts), eigenvalues
 * ascending; stands in for LAPACK dspevd (pCore-1.9.0/extensions/csource/LAPACKEigenvalueSolver.c:21). */
static void eigen(int n, double *a, double *w)
{
    /* a: n x n row-major symmetric in, eigenvectors in columns out */
    double *e = (double *)calloc(n, sizeof(double));
    for (int i = n - 1; i > 0; i--) {
        int l = i - 1;
        double h = 0.0, scale = 0.0;
        if (l > 0) {
            for (int k = 0; k <= l; k++) scale += fabs(a[i * n + k]);
            if (scale == 0.0) e[i] = a[i * n + l];
            else {
                for (int k = 0; k <= l; k++) { a[i * n + k] /= scale; h += a[i * n + k] * a[i * n + k]; }
                double f = a[i * n + l], g = (f >= 0.0) ? -sqrt(h) : sqrt(h);
                e[i] = scale * g; h -= f * g; a[i * n + l] = f - g; f = 0.0;
                for (int j = 0; j <= l; j++) {
                    a[j * n + i] = a[i * n + j] / h;
                    g = 0.0;
                    for (int k = 0; k <= j; k++) g += a[j * n + k] * a[i * n + k];
                    for (int k = j + 1; k <= l; k++) g += a[k * n + j] * a[i * n + k];
                    e[j] = g / h; f += e[j] * a[i * n + j];
                }
                double hh = f / (h + h);
                for (int j = 0; j <= l; j++) {
                    f = a[i * n + j]; e[j] = g = e[j] - hh * f;
                    for (int k = 0; k <= j; k++) a[j * n + k] -= (f * e[k] + g * a[i * n + k]);
                }
            }
        } else e[i] = a[i * n + l];
        w[i] = h;
    }
    w[0] = 0.0; e[0] = 0.0;
    for (int i = 0; i < n; i++) {
        int l = i - 1;
        if (w[i] != 0.0) {
            for (int j = 0; j <= l; j++) {
                double g = 0.0;
                for (int k = 0; k <= l; k++) g += a[i * n + k] * a[k * n + j];
                for (int k = 0; k <= l; k++) a[k * n + j] -= g * a[k * n + i];
            }
        }
        w[i] = a[i * n + i]; a[i * n + i] = 1.0;
        for (int j = 0; j <= l; j++) a[j * n + i] = a[i * n + j] = 0.0;
    }
    for (int i = 1; i < n; i++) e[i - 1] = e[i];
    e[n - 1] = 0.0;
    for (int l = 0; l < n; l++) {
        int iter = 0, m;
        do {
            for (m = l; m < n - 1; m++) {
                double dd = fabs(w[m]) + fabs(w[m + 1]);
                if (fabs(e[m]) <= 1.0e-15 * dd) break;
            }
            if (m != l) {
                if (iter++ == 60) break;
                double g = (w[l + 1] - w[l]) / (2.0 * e[l]);
                double r = hypot(g, 1.0);
                g = w[m] - w[l] + e[l] / (g + (g >= 0.0 ? fabs(r) : -fabs(r)));
                double s = 1.0, c = 1.0, p = 0.0;
                int i;
                for (i = m - 1; i >= l; i--) {
                    double f = s * e[i], b = c * e[i];
                    e[i + 1] = (r = hypot(f, g));
                    if (r == 0.0) { w[i + 1] -= p; e[m] = 0.0; break; }
                    s = f / r; c = g / r; g = w[i + 1] - p; r = (w[i] - g) * s + 2.0 * c * b;
                    w[i + 1] = g + (p = s * r); g = c * r - b;
                    for (int k = 0; k < n; k++) {
                        f = a[k * n + i + 1];
                        a[k * n + i + 1] = s * a[k * n + i] + c * f;
                        a[k * n + i] = c * a[k * n + i] - s * f;
                    }
                }
                if (r == 0.0 && i >= l) continue;
                w[l] -= p; e[l] = g; e[m] = 0.0;
            }
        } while (m != l);
    }
    for (int i = 0; i < n - 1; i++) {   /* sort ascending */
        int k = i; double p = w[i];
        for (int j = i + 1; j < n; j++) if (w[j] < p) { k = j; p = w[j]; }
        if (k != i) {
            w[k] = w[i]; w[i] = p;
            for (int j = 0; j < n; j++) { double t = a[j * n + i]; a[j * n + i] = a[j * n + k]; a[j * n + k] = t; }
        }
    }
    free(e);
}

/* Density from the Fock matrix: diagonalise, occupy the lowest nocc orbitals with 2 electrons,
 * P = sum 2 c c^T; returns the RMS difference ||P_new - P_old||_F / N over the packed
 * lower triangle as SymmetricMatrix_Trace2 defines it (csource/QCOnePDM.c:369-400,403-460).        */
static double density_from_fock(int N, int nocc, const double *F, double *P, double *work)
{
    memcpy(work, F, sizeof(double) * N * N);
    double *w = (double *)malloc(sizeof(double) * N);
    eigen(N, work, w);
    double rms = 0.0;
    for (int i = 0; i < N; i++)
        for (int j = 0; j <= i; j++) {
            double v = 0.0;
            for (int o = 0; o < nocc; o++) v += 2.0 * work[i * N + o] * work[j * N + o];
            double d = v - P[i * N + j];
            rms += (i == j) ? d * d : 2.0 * d * d;
            P[i * N + j] = P[j * N + i] = v;
        }
    free(w);
    return sqrt(rms) / (double)N;
}

/* tr(A B) over full symmetric matrices (SymmetricMatrix_Multiply2_Trace, SymmetricMatrix.c:856). */
static double trace2(int N, const double *A, const double *B)
{
    double t = 0.0;
    for (int i = 0; i < N * N; i++) t += A[i] * B[i];
    return t;
}

/* Small dense solve with partial pivoting; returns 0 on success, 1 if singular or ill-conditioned
 * (reciprocal 1-norm condition number below 1e-15, the test of SymmetricMatrix.c:1412-1450).      */
static int solve_small(int n, double *A, double *b)
{
    double Ainv[12][12], M[12][12], anorm = 0.0;
    for (int j = 0; j < n; j++) { double s = 0.0; for (int i = 0; i < n; i++) s += fabs(A[i * n + j]); if (s > anorm) anorm = s; }
    for (int i = 0; i < n; i++) for (int j = 0; j < n; j++) { M[i][j] = A[i * n + j]; Ainv[i][j] = (i == j); }
    double x[12]; for (int i = 0; i < n; i++) x[i] = b[i];
    for (int k = 0; k < n; k++) {
        int p = k; for (int i = k + 1; i < n; i++) if (fabs(M[i][k]) > fabs(M[p][k])) p = i;
        if (M[p][k] == 0.0) return 1;
        if (p != k) {
            for (int j = 0; j < n; j++) { double t = M[k][j]; M[k][j] = M[p][j]; M[p][j] = t; t = Ainv[k][j]; Ainv[k][j] = Ainv[p][j]; Ainv[p][j] = t; }
            double t = x[k]; x[k] = x[p]; x[p] = t;
        }
        for (int i = 0; i < n; i++) {
            if (i == k) continue;
            double f = M[i][k] / M[k][k];
            if (f == 0.0) continue;
            for (int j = 0; j < n; j++) { M[i][j] -= f * M[k][j]; Ainv[i][j] -= f * Ainv[k][j]; }
            x[i] -= f * x[k];
        }
    }
    double inorm = 0.0;
    for (int j = 0; j < n; j++) { double s = 0.0; for (int i = 0; i < n; i++) s += fabs(Ainv[i][j] / M[i][i]); if (s > inorm) inorm = s; }
    for (int i = 0; i < n; i++) b[i] = x[i] / M[i][i];
    if (!(anorm * inorm < 1.0e15)) return 1;
    return 0;
}

/* ================================================================================================ */
/* QC/MM: Lowdin charges q_A = Z_A - sum P_mm (csource/QCModelMNDO.c:1459-1520), energy q.phi and
 * -phi_A on the diagonal of the Fock matrix (:1808-1860).                                          */
static double qcmm_fock(const Config *c, const double *phi, const double *P, double *F, double *q)
{
    double e = 0.0;
    int N = c->nBasis;
    for (int i = 0; i < c->nAtoms; i++) {
        double ps = 0.0;
        for (int m = c->start[i]; m < c->start[i] + c->norb[i]; m++) ps += P[m * N + m];
        double qi = c->el[i]->zcore - ps;
        if (q) q[i] = qi;
        if (phi) {
            e += qi * phi[i];
            for (int m = c->start[i]; m < c->start[i] + c->norb[i]; m++) F[m * N + m] -= phi[i];
        }
    }
    return e;
}

/* One Fock build: F = H + G(P); QC electronic energy tr(PH) + tr(PG)/2 (csource/QCModelMNDO.c:700-730). */
static double build_fock(const Config *c, const double *P, double *F, const double *phi, double *q, double *eqc, double *eoei, double *etei)
{
    int N = c->nBasis;
    fock_g(c, P, F);
    double e1 = trace2(N, P, c->H), e2 = 0.5 * trace2(N, P, F);
    for (int i = 0; i < N * N; i++) F[i] += c->H[i];
    *eqc = e1 + e2; if (eoei) *eoei = e1; if (etei) *etei = e2;
    return qcmm_fock(c, phi, P, F, q);
}

/* ================================================================================================ */
/* Gradients: csource/QCModelMNDO.c:732-855 with csource/QCModelMNDOState.c:178-260 (density terms) and
 * csource/MNDOIntegrals.c:274-450 (MolecularFrame2CIntegralsD).  Output in Eh/Bohr.               */
static void gradients(const Config *c, const double *P, const double *S, double *g)
{
    int N = c->nBasis;
    memset(g, 0, sizeof(double) * 3 * c->nAtoms);
    for (int i = 0; i < c->nAtoms; i++)
        for (int j = 0; j < i; j++) {
            const Element *ei = c->el[i], *ej = c->el[j];
            int is = c->start[i], js = c->start[j];
            int ni = ei->norb * (ei->norb + 1) / 2, nj = ej->norb * (ej->norb + 1) / 2;
            double oneI[10] = {0}, oneJ[10] = {0}, gam[10][10];
            int ab = 0;
            for (int a = 0; a < ei->norb; a++) for (int b = 0; b <= a; b++, ab++) oneI[ab] = (a == b ? 1.0 : 2.0) * P[(is + a) * N + is + b];
            ab = 0;
            for (int a = 0; a < ej->norb; a++) for (int b = 0; b <= a; b++, ab++) oneJ[ab] = (a == b ? 1.0 : 2.0) * P[(js + a) * N + js + b];
            /* exchange part: 1/4 aa bb (P_mk P_nl + P_nk P_ml), k<=l on i, m<=n on j; minus Coulomb */
            for (int k = 0; k < ei->norb; k++)
                for (int l = k; l < ei->norb; l++) {
                    int kl = PK(l, k);
                    double aa = (k == l) ? 1.0 : 2.0;
                    for (int m = 0; m < ej->norb; m++)
                        for (int n = m; n < ej->norb; n++) {
                            int mn = PK(n, m);
                            double bb = (m == n) ? 1.0 : 2.0;
                            int K = is + k, Lx = is + l, M = js + m, Nn = js + n;
                            double f = P[M * N + K] * P[Nn * N + Lx] + P[Nn * N + K] * P[M * N + Lx];
                            /* open shell: the spin density's products join the exchange part
                               (csource/QCModelMNDOState.c:178-260, dspin) */
                            if (S) f += S[M * N + K] * S[Nn * N + Lx] + S[Nn * N + K] * S[M * N + Lx];
                            gam[kl][mn] = 0.25 * aa * bb * f - oneI[kl] * oneJ[mn];
                        }
                }
            double C[10][10], CD[3][10][10], v[3], L[10][10], LD[10][10], c1[10], d1[10], c2[10], d2[10];
            double r = rotation(c->xyz + 3 * i, c->xyz + 3 * j, ei->norb > ej->norb ? ei->norb : ej->norb, C, CD, v);
            double eng[3] = {0, 0, 0};
            if (r >= SMALL_RIJ) {
                local_teis(ei, ej, r, L, LD);
                local_core(ei, ej, r, 0, c1, d1);
                local_core(ej, ei, r, 1, c2, d2);
                double dcore;
                core_core(ei, ej, r, &dcore);
                /* radial parts */
                double doei0f = 0.0, dtei0f = 0.0;
                for (int a = 0; a < ni; a++) { double t = 0; for (int p = 0; p < ni; p++) t += C[a][p] * d1[p]; doei0f += oneI[a] * t; }
                for (int a = 0; a < nj; a++) { double t = 0; for (int p = 0; p < nj; p++) t += C[a][p] * d2[p]; doei0f += oneJ[a] * t; }
                for (int a = 0; a < ni; a++)
                    for (int b = 0; b < nj; b++) {
                        double t = 0;
                        for (int p = 0; p < ni; p++) for (int q = 0; q < nj; q++) t += C[a][p] * LD[p][q] * C[b][q];
                        dtei0f -= gam[a][b] * t;
                    }
                for (int x = 0; x < 3; x++) {
                    double s = v[x] / r;
                    double doei1 = 0.0, dtei1 = 0.0;
                    int doI = (ei->norb > 1), doJ = (ej->norb > 1);
                    int any = (ei->norb > 1 || ej->norb > 1);
                    /* rotation parts (only atoms with p orbitals have a non-identity transform) */
                    if (doI) for (int a = 0; a < ni; a++) { double t = 0; for (int p = 0; p < ni; p++) t += CD[x][a][p] * c1[p]; doei1 -= oneI[a] * t; }
                    if (doJ) for (int a = 0; a < nj; a++) { double t = 0; for (int p = 0; p < nj; p++) t += CD[x][a][p] * c2[p]; doei1 -= oneJ[a] * t; }
                    if (any && r * r > SMALL_RIJ2) {
                        for (int a = 0; a < ni; a++)
                            for (int b = 0; b < nj; b++) {
                                double t = 0;
                                for (int p = 0; p < ni; p++)
                                    for (int q = 0; q < nj; q++) {
                                        double ti = doI ? CD[x][a][p] * C[b][q] : 0.0;
                                        double tj = doJ ? C[a][p] * CD[x][b][q] : 0.0;
                                        t += (ti + tj) * L[p][q];
                                    }
                                dtei1 += gam[a][b] * t;
                            }
                    }
                    eng[x] = -s * dcore - s * doei0f + doei1 - s * dtei0f + dtei1;
                }
            }
            /* resonance integral derivatives: sum (beta_i + beta_j) P_ij dS_ij (implicit factor 2) */
            double S[4][4], SD[3][4][4];
            overlap(ei, c->xyz + 3 * i, ej, c->xyz + 3 * j, S, SD);
            for (int a = 0; a < ei->norb; a++)
                for (int b = 0; b < ej->norb; b++) {
                    double bp = (ei->beta[a] + ej->beta[b]) * P[(is + a) * N + js + b];
                    for (int x = 0; x < 3; x++) eng[x] += bp * SD[x][a][b];
                }
            for (int x = 0; x < 3; x++) { g[3 * i + x] += eng[x]; g[3 * j + x] -= eng[x]; }
        }
}

/* ================================================================================================ */
/* The SCF: QCModel.Energy (pMolecule.QCModel.pyx:146-185) driving DIISSCFConverger
 * (csource/DIISSCFConverger.c:100-130 Continue/Converged, :147-252 IterateWithoutDensities, :256-270
 * MakeDensities, :385-521 DIIS_Fock_Save, :530-650 DIIS_Iterate, :661-760 RCA_Iterate) with the
 * initial uniform diagonal guess (csource/QCOnePDM.c:280-345).                                     */
typedef struct {
    int n, ndiis, matnum, matind[16];
    double *xP[16], *xF[16], *err[16], b[16][16];
    double *rP, *rF;
} DIIS;

static double diis_save(DIIS *d, int N, const double *P, const double *F, double *work)
{
    int newest;
    if (d->matnum < d->ndiis) { d->matnum++; newest = d->matind[d->matnum - 1]; }
    else {
        d->matnum = d->ndiis; newest = d->matind[0];
        for (int i = 0; i < d->ndiis - 1; i++) d->matind[i] = d->matind[i + 1];
        d->matind[d->ndiis - 1] = newest;
    }
    memcpy(d->xP[newest], P, sizeof(double) * N * N);
    memcpy(d->xF[newest], F, sizeof(double) * N * N);
    /* e = F P - (F P)^T, strict lower triangle (AntisymmetricMatrix.c:159 CommutatorSS_Fast) */
    for (int i = 0; i < N; i++)
        for (int j = 0; j < N; j++) { double s = 0; for (int k = 0; k < N; k++) s += F[i * N + k] * P[k * N + j]; work[i * N + j] = s; }
    double *e = d->err[newest], emax = 0.0;
    int t = 0;
    for (int i = 0; i < N; i++)
        for (int j = 0; j < i; j++, t++) { e[t] = work[i * N + j] - work[j * N + i]; if (fabs(e[t]) > emax) emax = fabs(e[t]); }
    int ne = N * (N - 1) / 2;
    for (int m = 0; m < d->matnum; m++) {
        int n = d->matind[m];
        double s = 0.0;
        for (int k = 0; k < ne; k++) s += d->err[n][k] * e[k];
        double f = 2.0 * s;   /* - AntisymmetricMatrix_Trace2 = 2 e.e */
        d->b[n][newest] = f; if (n != newest) d->b[newest][n] = f;
    }
    return emax;
}

static void diis_iterate(DIIS *d, int N, double *P, double *F)
{
    if (d->matnum <= 1) return;
    double A[144], b[12];
    while (1) {
        int m = d->matnum, n = m + 1;
        for (int i = 0; i < n * n; i++) A[i] = 0.0;
        for (int i = 0; i < m; i++)
            for (int j = 0; j < m; j++) A[i * n + j] = d->b[d->matind[i]][d->matind[j]];
        for (int i = 0; i < m; i++) { A[m * n + i] = -1.0; A[i * n + m] = -1.0; }
        for (int i = 0; i < n; i++) b[i] = 0.0;
        b[m] = -1.0;
        int bad = solve_small(n, A, b);
        b[m] = -1.0;
        double dev = 0.0; for (int i = 0; i < n; i++) dev += b[i];
        if (!bad && fabs(dev) < 1.0e-6) break;
        d->matnum--;
        for (int i = 0; i < d->matnum; i++) d->matind[i] = d->matind[i + 1];
        for (int i = d->matnum; i < d->ndiis; i++) {
            d->matind[i] = d->matind[i - 1] + 1;
            if (d->matind[i] >= d->ndiis) d->matind[i] -= d->ndiis;
        }
        if (d->matnum <= 1) return;
    }
    memset(P, 0, sizeof(double) * N * N); memset(F, 0, sizeof(double) * N * N);
    for (int m = 0; m < d->matnum; m++) {
        int n = d->matind[m];
        for (int k = 0; k < N * N; k++) { P[k] += b[m] * d->xP[n][k]; F[k] += b[m] * d->xF[n][k]; }
    }
}

static void rca_iterate(DIIS *d, int N, double *P, double *F, double eold, double *energy)
{
    double a = trace2(N, F, P) - trace2(N, F, d->rP);
    double c = trace2(N, d->rF, P) - trace2(N, d->rF, d->rP);
    double dd = eold;
    a += c + 2.0 * (dd - *energy);
    double b = *energy - a - c - dd;
    double fmin = *energy, mubmin = 1.0, mu;
    if (eold < *energy) { fmin = eold; mubmin = 0.0; }
    if (a == 0.0) {
        if (b == 0.0) mu = mubmin;
        else { double mut = -c / (2.0 * b); mu = (b > 0.0 && mut > 0.0 && mut < 1.0) ? mut : mubmin; }
    } else {
        double fac = b * b - 3.0 * a * c;
        if (fac >= 0.0) {
            double m1 = (-b + sqrt(fac)) / (3.0 * a), m2 = (-b - sqrt(fac)) / (3.0 * a);
            if (m1 > 0.0 && m1 < 1.0) { double f = ((a * m1 + b) * m1 + c) * m1 + dd; if (f < fmin) { fmin = f; mubmin = m1; } }
            if (m2 > 0.0 && m2 < 1.0) { double f = ((a * m2 + b) * m2 + c) * m2 + dd; if (f < fmin) { fmin = f; mubmin = m2; } }
        }
        mu = mubmin;
    }
    if (mu < 0.01) mu = 0.01;
    double nu = 1.0 - mu;
    for (int k = 0; k < N * N; k++) { P[k] = mu * P[k] + nu * d->rP[k]; F[k] = mu * F[k] + nu * d->rF[k]; }
    *energy = ((a * mu + b) * mu + c) * mu + dd;
}

int oracle_energy(const OracleHamiltonian *h, int nAtoms, const int *elementIndex, const double *xyz, int charge,
                  const double *phi, const OracleSCFOptions *o, double *density, int useDensity,
                  double *energies, double *grad, double *charges, int *ncycles, double *oneElectron)
{
    if (!h || nAtoms <= 0 || !o) return 4;
    Config c;
    config_init(&c, h, nAtoms, elementIndex, xyz);
    integrals(&c);
    int N = c.nBasis, nz = 0;
    for (int i = 0; i < nAtoms; i++) nz += (int)lround(c.el[i]->zcore);
    int nel = nz - charge, nocc = (nel + 1) / 2;
    double *P = (double *)calloc((size_t)N * N, sizeof(double)), *F = (double *)calloc((size_t)N * N, sizeof(double));
    double *work = (double *)calloc((size_t)N * N, sizeof(double));
    if (useDensity && density) {
        for (int i = 0; i < N; i++) for (int j = 0; j <= i; j++) P[i * N + j] = P[j * N + i] = density[PK(i, j)];
    } else {
        for (int i = 0; i < N; i++) P[i * N + i] = (double)nel / (double)N;
    }
    if (oneElectron) for (int i = 0; i < N; i++) for (int j = 0; j <= i; j++) oneElectron[PK(i, j)] = c.H[i * N + j];
    DIIS d; memset(&d, 0, sizeof(d));
    d.ndiis = o->history;
    for (int i = 0; i < d.ndiis; i++) {
        d.matind[i] = i;
        d.xP[i] = (double *)calloc((size_t)N * N, sizeof(double));
        d.xF[i] = (double *)calloc((size_t)N * N, sizeof(double));
        d.err[i] = (double *)calloc((size_t)N * (N - 1) / 2 + 1, sizeof(double));
    }
    d.rP = (double *)calloc((size_t)N * N, sizeof(double)); d.rF = (double *)calloc((size_t)N * N, sizeof(double));
    int iteration = 0, converged = 0, qdiis = 0, qrca = o->useRCA ? 1 : 0, valid = (useDensity && density) ? 1 : 0;
    double eold = 0.0, deltaeold = 0.0, rms = 0.0, eqc = 0.0, eqcmm = 0.0, eoei = 0.0, etei = 0.0;
    while (iteration < o->maximumSCFCycles && !converged) {
        eqcmm = build_fock(&c, P, F, phi, charges, &eqc, &eoei, &etei);
        double eel = eqc + eqcmm;
        converged = (iteration > 0) && (rms <= o->densityTolerance) && (deltaeold <= o->energyTolerance);
        if (converged) break;
        double deltae = eel - eold, etemp = eel;
        /* the diagonal guess is not a valid density: its cycle is neither stored nor counted
           (DIISSCFConverger.c:160,240; QCOnePDM.c:390) */
        if (valid) {
            double maxerr = (N > 1) ? diis_save(&d, N, P, F, work) : 0.0;
            if (iteration > 0) {
                if (o->useRCA) {
                    if (qdiis && maxerr > 0.8) { qdiis = 0; qrca = 1; }
                    else if (iteration > 1 && qrca && maxerr < o->diisOnset) { qdiis = 1; qrca = 0; }
                }
                if (qdiis && N > 1) diis_iterate(&d, N, P, F);
                else if (o->useRCA && qrca) rca_iterate(&d, N, P, F, eold, &etemp);
            }
            if (o->useRCA) { memcpy(d.rP, P, sizeof(double) * N * N); memcpy(d.rF, F, sizeof(double) * N * N); }
            iteration++;
        }
        deltaeold = deltae; eold = etemp;
        rms = density_from_fock(N, nocc, F, P, work);
        valid = 1;
    }
    if (ncycles) *ncycles = iteration;
    energies[0] = eqc + eqcmm; energies[1] = eqc; energies[2] = c.enuc;
    double base = 0.0; for (int i = 0; i < nAtoms; i++) base += c.el[i]->eheat - c.el[i]->eisol;
    energies[3] = base; energies[4] = eqcmm; energies[5] = 0.0; energies[6] = eoei; energies[7] = etei;
    if (grad && converged) gradients(&c, P, NULL, grad);
    if (density) for (int i = 0; i < N; i++) for (int j = 0; j <= i; j++) density[PK(i, j)] = P[i * N + j];
    for (int i = 0; i < d.ndiis; i++) { free(d.xP[i]); free(d.xF[i]); free(d.err[i]); }
    free(d.rP); free(d.rF); free(P); free(F); free(work);
    config_free(&c);
    return converged ? 0 : 1;
}

/* ================================================================================================ */
/* Open-shell and fractional-occupancy states (QCModelMNDO keywords isSpinRestricted, occupancyType):
 * restricted densities hold the total density (occupancy factor 2), unrestricted ones alpha and beta
 * (factor 1) (csource/QCModelMNDOState.c QCModelMNDOState_Setup).                                   */

/* Two-electron part G = J(Pt) - K(Ps) of one spin's Fock matrix: Coulomb from the total density, exchange
 * from the density of that spin (csource/MNDOIntegrals.c:51-143 MakeFockG with its second density;
 * the one-centre terms split as (ss|ss) = gss, (ss|pp) = gsp, (sp|sp) = hsp, (pp|pp) = gpp,
 * (pp|qq) = gp2, (pq|pq) = hpp).  fock_g is the case Ps = Pt / 2.                                  */
static void fock_g_spin(const Config *c, const double *Pt, const double *Ps, double *G)
{
    int N = c->nBasis;
    memset(G, 0, sizeof(double) * N * N);
    for (int i = 0; i < c->nAtoms; i++) {
        const Element *e = c->el[i];
        int s = c->start[i];
        if (fabs(e->gss) > TEI_UNDERFLOW) G[s * N + s] += (Pt[s * N + s] - Ps[s * N + s]) * e->gss;
        if (e->norb == 4) {
            for (int p = 1; p < 4; p++) {
                int pp = s + p;
                G[s * N + s] += Pt[pp * N + pp] * e->gsp - Ps[pp * N + pp] * e->hsp;
                G[pp * N + pp] += Pt[s * N + s] * e->gsp - Ps[s * N + s] * e->hsp + (Pt[pp * N + pp] - Ps[pp * N + pp]) * e->gpp;
                double v = 2.0 * Pt[s * N + pp] * e->hsp - Ps[s * N + pp] * (e->hsp + e->gsp);
                G[s * N + pp] += v; G[pp * N + s] += v;
                for (int q = 1; q < 4; q++) {
                    if (q == p) continue;
                    int qq = s + q;
                    G[pp * N + pp] += Pt[qq * N + qq] * e->gp2 - Ps[qq * N + qq] * e->hpp;
                    G[pp * N + qq] += 2.0 * Pt[pp * N + qq] * e->hpp - Ps[pp * N + qq] * (e->hpp + e->gp2);
                }
            }
        }
        for (int j = 0; j < i; j++) {
            const double *blk = c->tei + (size_t)pair_index(i, j) * 100;
            int is = c->start[i], js = c->start[j], ni = c->norb[i], nj = c->norb[j];
            int ab = 0;
            for (int a = 0; a < ni; a++)
                for (int b = 0; b <= a; b++, ab++) {
                    int cd = 0;
                    for (int cc = 0; cc < nj; cc++)
                        for (int d = 0; d <= cc; d++, cd++) {
                            double v = blk[ab * 10 + cd];
                            if (fabs(v) <= TEI_UNDERFLOW) continue;
                            int A[2] = { is + a, is + b }, B[2] = { js + cc, js + d };
                            int na = (a == b) ? 1 : 2, nb = (cc == d) ? 1 : 2;
                            for (int u = 0; u < na; u++)
                                for (int w = 0; w < nb; w++) {
                                    int m = A[u], n = A[1 - u], l = B[w], sg = B[1 - w];
                                    if (na == 1) n = m;
                                    if (nb == 1) sg = l;
                                    G[m * N + n] += v * Pt[l * N + sg];
                                    G[l * N + sg] += v * Pt[m * N + n];
                                    G[m * N + l] -= v * Ps[n * N + sg];
                                    G[l * N + m] -= v * Ps[n * N + sg];
                                }
                        }
                }
        }
    }
}

/* Orbital occupancies of one density (csource/QCOnePDM.c:256-275 FermiOccupancies, :280-345
 * FromDiagonalGuess, :505-570 Occupancies, :572-599 OccupancyEnergy).                               */
typedef struct {
    int type, nOccupied, nOrbitals;
    double factor, charge, broadening, eocc, *occ;
} Occupancy;

static int occupancy_init(Occupancy *o, int type, double factor, double charge, int nHOO, int nLUO, int N, double broadening)
{
    memset(o, 0, sizeof(*o));
    o->type = type; o->factor = factor; o->charge = charge; o->broadening = broadening; o->nOrbitals = N;
    o->occ = (double *)calloc((size_t)N, sizeof(double));
    int nOcc = (int)lround(ceil(charge / factor)), nCard = 0, nFrac = 0;
    double frac = 0.0;
    int ok = 1;
    if (type == 0) { ok = fabs((double)nOcc * factor - charge) < 1.0e-10; nCard = nOcc; }
    else if (type == 1) {
        nCard = nOcc - nHOO; nFrac = nHOO + nLUO; nOcc = nCard + nFrac;
        frac = (charge / factor - (double)nCard) / (double)(nFrac > 1 ? nFrac : 1);
        ok = nHOO > 0 && nLUO >= 0 && nCard >= 0 && nCard + nFrac <= N && frac >= 0.0 && frac <= 1.0;
    }
    if (!ok || charge < 0.0) return 0;
    if (type != 2) {
        o->nOccupied = nOcc;
        for (int i = 0; i < nCard; i++) o->occ[i] = factor;
        for (int i = 0; i < nFrac; i++) o->occ[nCard + i] = frac * factor;
    }
    return 1;
}

static double fermi_occupancies(Occupancy *o, const double *w, double ef)
{
    double q = 0.0;
    for (int i = 0; i < o->nOrbitals; i++) {
        double e = -o->broadening * (ef - w[i]);
        o->occ[i] = (e > 500.0) ? 0.0 : (e < -500.0 ? 1.0 : 1.0 / (1.0 + exp(e)));
        q += o->occ[i];
    }
    return q;
}

static void occupancy_update(Occupancy *o, const double *w)
{
    o->eocc = 0.0;
    if (o->type != 2) return;
    double target = o->charge / o->factor;
    o->nOccupied = 0;
    for (int i = 0; i < o->nOrbitals; i++) o->occ[i] = 0.0;
    if (!(target > 0.0)) return;
    double lo = -1000.0, hi = 1000.0, fm = 0.0;
    fermi_occupancies(o, w, lo);
    fermi_occupancies(o, w, hi);
    double dx = hi - lo;
    for (int it = 0; it < 500; it++) {   /* bisection as the reference's (the upper bound is never moved) */
        dx *= 0.5;
        double ef = lo + dx;
        fm = fermi_occupancies(o, w, ef) - target;
        if (fm <= 0.0) lo = ef;
        if (fabs(fm) <= 1.0e-12) break;
    }
    double e = 0.0;
    for (int i = 0; i < o->nOrbitals; i++) {
        double p = o->occ[i], q = 1.0 - p;
        if (p > 1.0e-10) {
            o->nOccupied++;
            e += p * log(p);
            if (q > 1.0e-10) e += q * log(q);
        }
    }
    o->eocc = e / o->broadening;
    if (o->factor != 1.0) { o->eocc *= o->factor; for (int i = 0; i < o->nOrbitals; i++) o->occ[i] *= o->factor; }
}

/* Density from a Fock matrix with the occupancies (QCOnePDM_MakeFromFock, QCOnePDM.c:403-460 and
 * QCOnePDM_Make :369-400): P = sum over the first nOccupied orbitals of occ_i c_i c_i^T; returns the
 * RMS change as density_from_fock does.                                                             */
static double density_from_fock_occ(int N, Occupancy *o, const double *F, double *P, double *work)
{
    memcpy(work, F, sizeof(double) * N * N);
    double *w = (double *)malloc(sizeof(double) * N);
    eigen(N, work, w);
    occupancy_update(o, w);
    double rms = 0.0;
    for (int i = 0; i < N; i++)
        for (int j = 0; j <= i; j++) {
            double v = 0.0;
            for (int k = 0; k < o->nOccupied; k++) v += o->occ[k] * work[i * N + k] * work[j * N + k];
            double d = v - P[i * N + j];
            rms += (i == j) ? d * d : 2.0 * d * d;
            P[i * N + j] = P[j * N + i] = v;
        }
    free(w);
    return sqrt(rms) / (double)N;
}

/* DIIS / ODA over one or two density sets (DIISSCFConverger.c:385-528 with densityq, :530-650,
 * :661-760): B entries summed over the sets, the largest error doubled for two sets, every set
 * extrapolated or mixed with the same coefficients.                                                  */
typedef struct {
    int n, ndiis, matnum, matind[16], nsets;
    double *xP[2][16], *xF[2][16], *err[2][16], b[16][16];
    double *rP[2], *rF[2];
} DIIS2;

static double diis2_save(DIIS2 *d, int N, double *const *P, double *const *F, double *work)
{
    int newest;
    if (d->matnum < d->ndiis) { d->matnum++; newest = d->matind[d->matnum - 1]; }
    else {
        d->matnum = d->ndiis; newest = d->matind[0];
        for (int i = 0; i < d->ndiis - 1; i++) d->matind[i] = d->matind[i + 1];
        d->matind[d->ndiis - 1] = newest;
    }
    double emax = 0.0;
    int ne = N * (N - 1) / 2;
    for (int s = 0; s < d->nsets; s++) {
        memcpy(d->xP[s][newest], P[s], sizeof(double) * N * N);
        memcpy(d->xF[s][newest], F[s], sizeof(double) * N * N);
        for (int i = 0; i < N; i++)
            for (int j = 0; j < N; j++) { double t = 0; for (int k = 0; k < N; k++) t += F[s][i * N + k] * P[s][k * N + j]; work[i * N + j] = t; }
        double *e = d->err[s][newest];
        int t = 0;
        for (int i = 0; i < N; i++)
            for (int j = 0; j < i; j++, t++) { e[t] = work[i * N + j] - work[j * N + i]; if (fabs(e[t]) > emax) emax = fabs(e[t]); }
        for (int m = 0; m < d->matnum; m++) {
            int n = d->matind[m];
            double x = 0.0;
            for (int k = 0; k < ne; k++) x += d->err[s][n][k] * e[k];
            double f = 2.0 * x;
            if (s == 0) { d->b[n][newest] = f; if (n != newest) d->b[newest][n] = f; }
            else { d->b[n][newest] += f; if (n != newest) d->b[newest][n] += f; }
        }
    }
    return d->nsets == 2 ? 2.0 * emax : emax;
}

static void diis2_iterate(DIIS2 *d, int N, double **P, double **F)
{
    if (d->matnum <= 1) return;
    double A[144], b[12];
    while (1) {
        int m = d->matnum, n = m + 1;
        for (int i = 0; i < n * n; i++) A[i] = 0.0;
        for (int i = 0; i < m; i++)
            for (int j = 0; j < m; j++) A[i * n + j] = d->b[d->matind[i]][d->matind[j]];
        for (int i = 0; i < m; i++) { A[m * n + i] = -1.0; A[i * n + m] = -1.0; }
        for (int i = 0; i < n; i++) b[i] = 0.0;
        b[m] = -1.0;
        int bad = solve_small(n, A, b);
        b[m] = -1.0;
        double dev = 0.0; for (int i = 0; i < n; i++) dev += b[i];
        if (!bad && fabs(dev) < 1.0e-6) break;
        d->matnum--;
        for (int i = 0; i < d->matnum; i++) d->matind[i] = d->matind[i + 1];
        for (int i = d->matnum; i < d->ndiis; i++) {
            d->matind[i] = d->matind[i - 1] + 1;
            if (d->matind[i] >= d->ndiis) d->matind[i] -= d->ndiis;
        }
        if (d->matnum <= 1) return;
    }
    for (int s = 0; s < d->nsets; s++) {
        memset(P[s], 0, sizeof(double) * N * N); memset(F[s], 0, sizeof(double) * N * N);
        for (int m = 0; m < d->matnum; m++) {
            int n = d->matind[m];
            for (int k = 0; k < N * N; k++) { P[s][k] += b[m] * d->xP[s][n][k]; F[s][k] += b[m] * d->xF[s][n][k]; }
        }
    }
}

static void rca2_iterate(DIIS2 *d, int N, double **P, double **F, double eold, double *energy)
{
    double a = 0.0, c = 0.0;
    for (int s = 0; s < d->nsets; s++) {
        a += trace2(N, F[s], P[s]) - trace2(N, F[s], d->rP[s]);
        c += trace2(N, d->rF[s], P[s]) - trace2(N, d->rF[s], d->rP[s]);
    }
    double dd = eold;
    a += c + 2.0 * (dd - *energy);
    double b = *energy - a - c - dd;
    double fmin = *energy, mubmin = 1.0, mu;
    if (eold < *energy) { fmin = eold; mubmin = 0.0; }
    if (a == 0.0) {
        if (b == 0.0) mu = mubmin;
        else { double mut = -c / (2.0 * b); mu = (b > 0.0 && mut > 0.0 && mut < 1.0) ? mut : mubmin; }
    } else {
        double fac = b * b - 3.0 * a * c;
        if (fac >= 0.0) {
            double m1 = (-b + sqrt(fac)) / (3.0 * a), m2 = (-b - sqrt(fac)) / (3.0 * a);
            if (m1 > 0.0 && m1 < 1.0) { double f = ((a * m1 + b) * m1 + c) * m1 + dd; if (f < fmin) { fmin = f; mubmin = m1; } }
            if (m2 > 0.0 && m2 < 1.0) { double f = ((a * m2 + b) * m2 + c) * m2 + dd; if (f < fmin) { fmin = f; mubmin = m2; } }
        }
        mu = mubmin;
    }
    if (mu < 0.01) mu = 0.01;
    double nu = 1.0 - mu;
    for (int s = 0; s < d->nsets; s++)
        for (int k = 0; k < N * N; k++) { P[s][k] = mu * P[s][k] + nu * d->rP[s][k]; F[s][k] = mu * F[s][k] + nu * d->rF[s][k]; }
    *energy = ((a * mu + b) * mu + c) * mu + dd;
}

/* The QC energy and gradients of an open-shell or fractional-occupancy state (QC only), as the reference
 * computes it (QCModelMNDO_Fock, QCModelMNDO.c: eelectronic = eocc + eoei + etei summed over the density
 * sets).  alphaCharge / betaCharge: QCModel.CrossCheckModelAndState (pMolecule.QCModel.pyx:99-118);
 * nFractional: (HOOs, LUOs, alpha HOOs, alpha LUOs, beta HOOs, beta LUOs).  energies as oracle_energy
 * (eocc in [5]); densityA / densityB (packed): total density when restricted (densityB untouched),
 * else alpha and beta.                                                                               */
int oracle_energy_open(const OracleHamiltonian *h, int nAtoms, const int *elementIndex, const double *xyz,
                       double alphaCharge, double betaCharge, int restricted, int occupancyType, const int *nFractional,
                       double fermiBroadening, const double *phi, const OracleSCFOptions *o, double *energies, double *grad,
                       double *charges, double *densityA, double *densityB, int *ncycles, const double *startA,
                       const double *startB)
{
    if (!h || nAtoms <= 0 || !o || !nFractional || occupancyType < 0 || occupancyType > 2) return 4;
    Config c;
    config_init(&c, h, nAtoms, elementIndex, xyz);
    integrals(&c);
    int N = c.nBasis, ns = restricted ? 1 : 2;
    Occupancy occ[2];
    memset(occ, 0, sizeof(occ));
    int ok = restricted ? occupancy_init(&occ[0], occupancyType, 2.0, alphaCharge + betaCharge, nFractional[0], nFractional[1], N, fermiBroadening)
                        : occupancy_init(&occ[0], occupancyType, 1.0, alphaCharge, nFractional[2], nFractional[3], N, fermiBroadening) &&
                          occupancy_init(&occ[1], occupancyType, 1.0, betaCharge, nFractional[4], nFractional[5], N, fermiBroadening);
    if (!ok) { for (int s = 0; s < ns; s++) free(occ[s].occ); config_free(&c); return 4; }
    double *P[2] = {NULL, NULL}, *F[2] = {NULL, NULL}, *G = (double *)calloc((size_t)N * N, sizeof(double));
    double *Pt = (double *)calloc((size_t)N * N, sizeof(double)), *Ps = (double *)calloc((size_t)N * N, sizeof(double));
    double *work = (double *)calloc((size_t)N * N, sizeof(double));
    for (int s = 0; s < ns; s++) {
        P[s] = (double *)calloc((size_t)N * N, sizeof(double)); F[s] = (double *)calloc((size_t)N * N, sizeof(double));
        for (int i = 0; i < N; i++) P[s][i * N + i] = occ[s].charge / (double)N;   /* diagonal guess (QCOnePDM.c:330) */
    }
    /* given start densities (packed; total density when restricted): used as a valid density, whose Fock matrices
       enter the DIIS history from the first cycle */
    const double *start[2] = { startA, startB };
    int valid = 0;
    if (startA && (restricted || startB)) {
        for (int s = 0; s < ns; s++)
            for (int i = 0; i < N; i++) for (int j = 0; j <= i; j++) P[s][i * N + j] = P[s][j * N + i] = start[s][PK(i, j)];
        valid = 1;
    }
    DIIS2 d; memset(&d, 0, sizeof(d));
    d.ndiis = o->history; d.nsets = ns;
    for (int i = 0; i < d.ndiis; i++) {
        d.matind[i] = i;
        for (int s = 0; s < ns; s++) {
            d.xP[s][i] = (double *)calloc((size_t)N * N, sizeof(double));
            d.xF[s][i] = (double *)calloc((size_t)N * N, sizeof(double));
            d.err[s][i] = (double *)calloc((size_t)N * (N - 1) / 2 + 1, sizeof(double));
        }
    }
    for (int s = 0; s < ns; s++) { d.rP[s] = (double *)calloc((size_t)N * N, sizeof(double)); d.rF[s] = (double *)calloc((size_t)N * N, sizeof(double)); }
    int iteration = 0, converged = 0, qdiis = 0, qrca = o->useRCA ? 1 : 0;
    double eold = 0.0, deltaeold = 0.0, rms = 0.0, eqc = 0.0, eoei = 0.0, etei = 0.0, eocc = 0.0, eqcmm = 0.0;
    while (iteration < o->maximumSCFCycles && !converged) {
        /* Fock matrices and energies (QCModelMNDO_Fock) */
        for (int k = 0; k < N * N; k++) Pt[k] = restricted ? P[0][k] : P[0][k] + P[1][k];
        eoei = etei = 0.0;
        eocc = occ[0].eocc + (ns == 2 ? occ[1].eocc : 0.0);
        for (int s = 0; s < ns; s++) {
            if (restricted) for (int k = 0; k < N * N; k++) Ps[k] = 0.5 * P[0][k];
            fock_g_spin(&c, Pt, restricted ? Ps : P[s], G);
            eoei += trace2(N, P[s], c.H);
            etei += 0.5 * trace2(N, P[s], G);
            for (int k = 0; k < N * N; k++) F[s][k] = G[k] + c.H[k];
        }
        eqc = eocc + eoei + etei;
        /* QC/MM: Lowdin charges of the total density, -phi on the diagonal of every spin's Fock matrix
           (QCModelMNDO_QCMMFockLowdin, QCModelMNDO.c) */
        eqcmm = 0.0;
        if (phi) {
            eqcmm = qcmm_fock(&c, phi, Pt, F[0], charges);
            if (ns == 2) qcmm_fock(&c, phi, Pt, F[1], NULL);
        }
        double eel = eqc + eqcmm;
        converged = (iteration > 0) && (rms <= o->densityTolerance) && (deltaeold <= o->energyTolerance);
        if (converged) break;
        double deltae = eel - eold, etemp = eel;
        if (valid) {
            double maxerr = (N > 1) ? diis2_save(&d, N, P, F, work) : 0.0;
            if (iteration > 0) {
                if (o->useRCA) {
                    if (qdiis && maxerr > 0.8) { qdiis = 0; qrca = 1; }
                    else if (iteration > 1 && qrca && maxerr < o->diisOnset) { qdiis = 1; qrca = 0; }
                }
                if (qdiis && N > 1) diis2_iterate(&d, N, P, F);
                else if (o->useRCA && qrca) rca2_iterate(&d, N, P, F, eold, &etemp);
            }
            if (o->useRCA)
                for (int s = 0; s < ns; s++) { memcpy(d.rP[s], P[s], sizeof(double) * N * N); memcpy(d.rF[s], F[s], sizeof(double) * N * N); }
            iteration++;
        }
        deltaeold = deltae; eold = etemp;
        rms = 0.0;
        for (int s = 0; s < ns; s++) { double r = density_from_fock_occ(N, &occ[s], F[s], P[s], work); if (r > rms) rms = r; }
        valid = 1;
    }
    if (ncycles) *ncycles = iteration;
    energies[0] = eqc + eqcmm; energies[1] = eqc; energies[2] = c.enuc;
    double base = 0.0; for (int i = 0; i < nAtoms; i++) base += c.el[i]->eheat - c.el[i]->eisol;
    energies[3] = base; energies[4] = eqcmm; energies[5] = eocc; energies[6] = eoei; energies[7] = etei;
    if (grad && converged) {
        for (int k = 0; k < N * N; k++) { Pt[k] = restricted ? P[0][k] : P[0][k] + P[1][k]; Ps[k] = restricted ? 0.0 : P[0][k] - P[1][k]; }
        gradients(&c, Pt, restricted ? NULL : Ps, grad);
    }
    for (int s = 0; s < ns; s++) {
        double *out = s == 0 ? densityA : densityB;
        if (out) for (int i = 0; i < N; i++) for (int j = 0; j <= i; j++) out[PK(i, j)] = P[s][i * N + j];
    }
    for (int i = 0; i < d.ndiis; i++) for (int s = 0; s < ns; s++) { free(d.xP[s][i]); free(d.xF[s][i]); free(d.err[s][i]); }
    for (int s = 0; s < ns; s++) { free(d.rP[s]); free(d.rF[s]); free(P[s]); free(F[s]); free(occ[s].occ); }
    free(G); free(Pt); free(Ps); free(work);
    config_free(&c);
    return converged ? 0 : 1;
}

int oracle_fock(const OracleHamiltonian *h, int nAtoms, const int *elementIndex, const double *xyz,
                const double *phi, const double *density, double *fock, double *energies)
{
    Config c;
    config_init(&c, h, nAtoms, elementIndex, xyz);
    integrals(&c);
    int N = c.nBasis;
    double *P = (double *)calloc((size_t)N * N, sizeof(double)), *F = (double *)calloc((size_t)N * N, sizeof(double)), eqc;
    for (int i = 0; i < N; i++) for (int j = 0; j <= i; j++) P[i * N + j] = P[j * N + i] = density[PK(i, j)];
    double eq = build_fock(&c, P, F, phi, NULL, &eqc, NULL, NULL);
    for (int i = 0; i < N; i++) for (int j = 0; j <= i; j++) fock[PK(i, j)] = F[i * N + j];
    energies[0] = eqc + eq; energies[1] = eqc; energies[2] = c.enuc;
    free(P); free(F); config_free(&c);
    return 0;
}

int oracle_gradients(const OracleHamiltonian *h, int nAtoms, const int *elementIndex, const double *xyz,
                     const double *density, double *g)
{
    Config c;
    config_init(&c, h, nAtoms, elementIndex, xyz);
    int N = c.nBasis;
    double *P = (double *)malloc(sizeof(double) * N * N);
    for (int i = 0; i < N; i++) for (int j = 0; j <= i; j++) P[i * N + j] = P[j * N + i] = density[PK(i, j)];
    gradients(&c, P, NULL, g);
    free(P); config_free(&c);
    return 0;
}

/* ================================================================================================ */
/* ABFS Delta/Gaussian spline for QC/MM (pMolecule.PairwiseInteraction.pyx:27-112,183-215 with
 * pCore/NumericalIntegration.py:21-65 AdaptiveSimpsonsRule), natural-derivative cubic spline in r^2
 * with zero end slopes (pCore-1.9.0/extensions/csource/CubicSpline.c MakeFromReal1DArrays, Evaluate:88). */
static double f_gauss(double p, double r)
{
    double x = p * r, x2 = x * x, f;
    if (x > 1.0e-2) f = erf(x) / x;
    else f = (2.0 - x2 * (2.0 / 3.0 - x2 * (0.2 - x2 * (1.0 / 21.0 - x2 * (1.0 / 108.0 - x2 / 660.0))))) / sqrt(PI);
    return f * p;
}

static double g_gauss(double p, double r)
{
    double sp = sqrt(PI), x = p * r, x2 = x * x, g;
    if (x > 1.0e-2) g = 2.0 * exp(-x2) / (sp * x) - erf(x) / x2;
    else g = -x * (4.0 / 3.0 - x2 * (0.8 - x2 * (2.0 / 7.0 - x2 * (2.0 / 27.0 - x2 / 66.0)))) / sp;
    return g * p * p;
}

static double switch_fn(double r, double on, double off)
{
    return pow(off * off - r * r, 2) * (off * off + 2.0 * r * r - 3.0 * on * on) / pow(off * off - on * on, 3);
}

static double gs(double p, double on, double off, double r) { return g_gauss(p, r) * switch_fn(r, on, off); }

typedef struct { double err, h, p0, p2, p4, f0, f2, f4, whole; } Interval;

static int iv_less(const Interval *a, const Interval *b)
{
    if (a->err != b->err) return a->err < b->err;
    if (a->h != b->h) return a->h < b->h;
    return a->p0 < b->p0;
}

static void heap_push(Interval *hp, int *n, Interval v)
{
    int i = (*n)++;
    hp[i] = v;
    while (i > 0) { int p = (i - 1) / 2; if (!iv_less(&hp[i], &hp[p])) break; Interval t = hp[i]; hp[i] = hp[p]; hp[p] = t; i = p; }
}

static Interval heap_pop(Interval *hp, int *n)
{
    Interval top = hp[0];
    hp[0] = hp[--(*n)];
    int i = 0;
    for (;;) {
        int l = 2 * i + 1, r = l + 1, m = i;
        if (l < *n && iv_less(&hp[l], &hp[m])) m = l;
        if (r < *n && iv_less(&hp[r], &hp[m])) m = r;
        if (m == i) break;
        Interval t = hp[i]; hp[i] = hp[m]; hp[m] = t; i = m;
    }
    return top;
}

static double adaptive_simpson(double p, double on, double off, double a, double b, double tol, int maxit)
{
    double h0 = fabs(a - b), eps = tol / h0, integral = 0.0;
    Interval *hp = (Interval *)malloc(sizeof(Interval) * (2 * maxit + 4));
    int n = 0, it = 0;
    double p1 = 0.5 * (a + b), f0 = gs(p, on, off, a), f1 = gs(p, on, off, p1), f2 = gs(p, on, off, b);
    Interval v0 = { 0.0, h0, a, p1, b, f0, f1, f2, (f0 + 4.0 * f1 + f2) * h0 / 6.0 };
    heap_push(hp, &n, v0);
    while (it < maxit && n > 0) {
        Interval v = heap_pop(hp, &n);
        double q1 = 0.5 * (v.p0 + v.p2), q3 = 0.5 * (v.p2 + v.p4);
        double g1 = gs(p, on, off, q1), g3 = gs(p, on, off, q3);
        double left = (v.f0 + 4.0 * g1 + v.f2) * v.h / 12.0, right = (v.f2 + 4.0 * g3 + v.f4) * v.h / 12.0;
        double lrw = left + right - v.whole, err = fabs(lrw);
        if (err < 15.0 * v.h * eps) integral += left + right + lrw / 15.0;
        else {
            double hh = 0.5 * v.h;
            Interval l = { -err, hh, v.p0, q1, v.p2, v.f0, g1, v.f2, left }, rr = { -err, hh, v.p2, q3, v.p4, v.f2, g3, v.f4, right };
            heap_push(hp, &n, l); heap_push(hp, &n, rr);
        }
        it++;
    }
    for (int i = 0; i < n; i++) integral += hp[i].whole;
    free(hp);
    if (a > b) integral = -integral;
    return integral;
}

int oracle_abfs_knots(double on, double off, double width2, int density, int maxKnots, double *x, double *y)
{
    double p = (2.0 / sqrt(PI)) / width2;
    int n = (int)ceil((double)density * off + 1.0);
    if (n > maxKnots) return -1;
    double inc = off / (double)(n - 1);
    x[0] = 0.0;
    for (int i = 1; i < n - 1; i++) x[i] = inc * (double)i;
    x[n - 1] = off;
    double integral = 0.0;
    int iupper = n - 2;
    y[n - 1] = 0.0;
    for (int i = n - 2; i >= 0; i--) {
        double lo = x[i], up = x[i + 1];
        if (lo < on) {
            iupper = i;
            if (up > on) integral -= adaptive_simpson(p, on, off, on, up, 1.0e-15, 1000);
            break;
        }
        integral -= adaptive_simpson(p, on, off, lo, up, 1.0e-15, 1000);
        y[i] = integral;
    }
    double offset = integral - f_gauss(p, on);
    for (int i = 0; i <= iupper; i++) y[i] = f_gauss(p, x[i]) + offset;   /* no damping for QC/MM */
    for (int i = 0; i < n; i++) { x[i] = x[i] * x[i]; y[i] /= ANGSTROMS_TO_BOHRS; }
    return n;
}

static void spline_second_derivatives(int n, const double *x, const double *y, double *hh)
{
    /* clamped (zero first derivative) ends, tridiagonal solve by elimination */
    double *dg = (double *)malloc(sizeof(double) * n), *sub = (double *)malloc(sizeof(double) * n), *sup = (double *)malloc(sizeof(double) * n);
    double dl = x[1] - x[0];
    dg[0] = dl / 3.0; sup[0] = dl / 6.0; hh[0] = (y[1] - y[0]) / dl;
    for (int i = 1; i < n - 1; i++) {
        dl = x[i] - x[i - 1]; double du = x[i + 1] - x[i];
        sub[i - 1] = dl / 6.0; dg[i] = (dl + du) / 3.0; sup[i] = du / 6.0;
        hh[i] = (y[i + 1] - y[i]) / du + (y[i - 1] - y[i]) / dl;
    }
    double du = x[n - 1] - x[n - 2];
    sub[n - 2] = du / 6.0; dg[n - 1] = du / 3.0; hh[n - 1] = -(y[n - 1] - y[n - 2]) / du;
    for (int i = 1; i < n; i++) { double m = sub[i - 1] / dg[i - 1]; dg[i] -= m * sup[i - 1]; hh[i] -= m * hh[i - 1]; }
    hh[n - 1] /= dg[n - 1];
    for (int i = n - 2; i >= 0; i--) hh[i] = (hh[i] - sup[i] * hh[i + 1]) / dg[i];
    free(dg); free(sub); free(sup);
}

static void spline_eval(int n, const double *x, const double *y, const double *hh, double v, double *f, double *g)
{
    int l = 0, u = n - 1;
    while (u - l > 1) { int i = (u + l) >> 1; if (x[i] > v) u = i; else l = i; }
    double d = x[u] - x[l], s = (v - x[l]) / d, t = (x[u] - v) / d;
    double hl = hh[l] * d / 6.0, hu = hh[u] * d / 6.0;
    *f = t * y[l] + s * y[u] + d * (t * (t * t - 1.0) * hl + s * (s * s - 1.0) * hu);
    *g = (y[u] - y[l]) / d + (-(3.0 * t * t - 1.0) * hl + (3.0 * s * s - 1.0) * hu);
}

int oracle_qcmm(int model, double on, double off, int nk, const double *x, const double *y,
                int nQC, const double *qcxyz, int nMM, const double *mmxyz, const double *mmq,
                const double *qcq, double *phi, double *gq, double *gm)
{
    (void)on;
    double *hh = NULL;
    if (model == 1) { hh = (double *)malloc(sizeof(double) * nk); spline_second_derivatives(nk, x, y, hh); }
    double r2off = off * off;
    if (gq) memset(gq, 0, sizeof(double) * 3 * nQC);
    if (gm) memset(gm, 0, sizeof(double) * 3 * nMM);
    for (int a = 0; a < nQC; a++) {
        double pot = 0.0;
        for (int m = 0; m < nMM; m++) {
            double d[3] = { qcxyz[3 * a] - mmxyz[3 * m], qcxyz[3 * a + 1] - mmxyz[3 * m + 1], qcxyz[3 * a + 2] - mmxyz[3 * m + 2] };
            double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2], f, dfdr2;
            if (model == 1) {
                if (r2 > r2off) continue;
                spline_eval(nk, x, y, hh, r2, &f, &dfdr2);               /* f a.u. per e; r^2 in A^2 */
            } else {
                double r = sqrt(r2);
                f = 1.0 / (r * ANGSTROMS_TO_BOHRS);
                dfdr2 = -0.5 / (r2 * r * ANGSTROMS_TO_BOHRS);
            }
            pot += mmq[m] * f;
            if (gq && qcq) {
                /* dE/dx (Eh/A) = q_a q_m 2 f'(r^2) dx ; converted to Eh/Bohr */
                double s = 2.0 * qcq[a] * mmq[m] * dfdr2 / ANGSTROMS_TO_BOHRS;
                for (int k = 0; k < 3; k++) { gq[3 * a + k] += s * d[k]; gm[3 * m + k] -= s * d[k]; }
            }
        }
        phi[a] = pot;
    }
    free(hh);
    return 0;
}
