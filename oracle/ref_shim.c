/*
 * ref_shim.c - test infrastructure: a C driver for pDynamo 1.9.0's own compiled C core.
 *
 * pDynamo's NDDO energy + gradient path is C (pMolecule-1.9.0/extensions/csource) driven by
 * Python-2 Pyrex glue that cannot run here.  This file restates that glue in C so that the
 * unmodified C core (linked into _ref/libpdynref.so by the Makefile in this directory) can be
 * run on the same inputs as the CUDA path.  It is a checker: only tests and the CPU-baseline
 * leg of bench.py load it.
 *
 * Restated glue, with the reference lines it follows:
 *   parameter load + unit conversion  pMolecule.MNDOParameters.pyx:140-207 (__setstate__),
 *                                      :212-275 (FillBetaUspd, FillFN123, FillPDDG), :309-370 (ToAtomicUnits)
 *   orbital basis load + scaling       pMolecule.GaussianBasis.pyx:96-122, pMolecule.QCParameters.pyx:131-140,188-200
 *   QC atom container                  pMolecule.QCAtomContainer.pyx:218-278
 *   model state set-up                 pMolecule.QCModelMNDO.pyx:623-672 (closed-shell RHF, cardinal occupancies)
 *   SCF loop                           pMolecule.QCModel.pyx:146-185, pMolecule.DIISSCFConverger.pyx:93-125
 *   energies                           pMolecule.QCModelMNDOState.pyx:168-185
 *   QC/MM electrostatics               pMolecule.NBModelABFS.pyx:124-138 over PairwiseInteraction.c:542,612
 *   MM/MM and QC/MM LJ energies        pMolecule.NBModelABFS.pyx:59-82,108-122 (generator and pairwise-interaction
 *                                      defaults, Energy), NBModelABFS.c:228-330 (MMMMEnergy, QCMMEnergyLJ) and
 *                                      :1050-1140 (GenerateLists, GenerateLists14), NBModelABFSState.c:207-226 (grids)
 */
# include <math.h>
# include <stdlib.h>
# include <string.h>

# include "BlockStorage.h"
# include "Coordinates3.h"
# include "CubicSpline.h"
# include "LJParameterContainer.h"
# include "MMAtomContainer.h"
# include "PairListGenerator.h"
# include "RegularGrid.h"
# include "RegularGridOccupancy.h"
# include "Selection.h"
# include "Vector3.h"
# include "DIISSCFConverger.h"
# include "DIISSCFConvergerState.h"
# include "GaussianBasis.h"
# include "GaussianBasisCore.h"
# include "MNDOParameters.h"
# include "PairList.h"
# include "PairwiseInteraction.h"
# include "QCAtomContainer.h"
# include "QCMMInteractionState.h"
# include "QCModelMNDO.h"
# include "QCModelMNDOState.h"
# include "QCOnePDM.h"
# include "QCParameters.h"
# include "Real1DArray.h"
# include "SymmetricMatrix.h"
# include "Units.h"

/* . pMolecule.MNDOParameters.pyx:18-21. */
# define BOHRS_TO_ANGSTROMS  UNITS_LENGTH_BOHRS_TO_ANGSTROMS
# define HARTREES_TO_EV      27.2113834e+00
# define HARTREES_TO_KCAL    ( 27.2113834e+00 * 23.060529e+00 )

/* . Order of the raw (file-unit) scalar parameters passed in by the caller. */
enum { R_III, R_IIID, R_IR016, R_IR066, R_IR244, R_IR266, R_IR466, R_QND, R_QNP, R_QNS,
       R_AD, R_ALP, R_AM, R_AQ, R_BETAD, R_BETAP, R_BETAS, R_DD, R_EHEAT, R_EISOL, R_F0SD, R_GPHOT,
       R_GPP, R_GP2, R_GSP, R_GSS, R_G2SD, R_HSP, R_PCORE, R_QQ, R_UDD, R_UPP, R_USS, R_ZCORE,
       R_ZETAD, R_ZETAP, R_ZETAS, R_ZDN, R_ZPN, R_ZSN, NRAW } ;
# define MAXGAUSS 4
# define MAXPDDG  4
# define MAXPRIM  6
# define MAXDIATOMIC 100

typedef struct {
    int          nElements ;
    int         *atomicNumbers ;
    QCParameter *parameters ;
} RefHamiltonian ;

typedef struct {
    RefHamiltonian       *hamiltonian ;
    int                   nAtoms ;
    QCAtomContainer      *qcAtoms ;
    QCModelMNDO          *model ;
    QCModelMNDOState     *state ;
    DIISSCFConverger     *converger ;
    Coordinates3         *coordinates3 ;
    Coordinates3         *gradients3 ;
    QCMMInteractionState *qcmm ;
} RefSystem ;

/* . Unit conversion of one element, pMolecule.MNDOParameters.pyx:212-275 and 309-370. */
static MNDOParameters *MakeElement ( const int atomicNumber, const int norbitals, const double *raw,
                                     const int nGaussians, const double *gaussians, const int nPDDG, const double *pddg,
                                     const int nDiatomic, const double *diatomic )
{
    int i ;
    MNDOParameters *p = MNDOParameters_Allocate ( ) ;
    p->atomicNumber = atomicNumber ; p->norbitals = norbitals ;
    p->iii   = ( int ) raw[R_III  ] ; p->iiid  = ( int ) raw[R_IIID ] ;
    p->ir016 = ( int ) raw[R_IR016] ; p->ir066 = ( int ) raw[R_IR066] ; p->ir244 = ( int ) raw[R_IR244] ;
    p->ir266 = ( int ) raw[R_IR266] ; p->ir466 = ( int ) raw[R_IR466] ;
    p->qnd   = ( int ) raw[R_QND  ] ; p->qnp   = ( int ) raw[R_QNP  ] ; p->qns = ( int ) raw[R_QNS] ;
    p->ad0 = raw[R_AD] ; p->alp0 = raw[R_ALP] ; p->am0 = raw[R_AM] ; p->aq0 = raw[R_AQ] ;
    p->betad0 = raw[R_BETAD] ; p->betap0 = raw[R_BETAP] ; p->betas0 = raw[R_BETAS] ; p->dd0 = raw[R_DD] ;
    p->eheat0 = raw[R_EHEAT] ; p->eisol0 = raw[R_EISOL] ; p->f0sd0 = raw[R_F0SD] ; p->gphot0 = raw[R_GPHOT] ;
    p->gpp0 = raw[R_GPP] ; p->gp20 = raw[R_GP2] ; p->gsp0 = raw[R_GSP] ; p->gss0 = raw[R_GSS] ; p->g2sd0 = raw[R_G2SD] ;
    p->hsp0 = raw[R_HSP] ; p->pcore0 = raw[R_PCORE] ; p->qq0 = raw[R_QQ] ; p->udd0 = raw[R_UDD] ; p->upp0 = raw[R_UPP] ;
    p->uss0 = raw[R_USS] ; p->zcore0 = raw[R_ZCORE] ; p->zetad0 = raw[R_ZETAD] ; p->zetap0 = raw[R_ZETAP] ;
    p->zetas0 = raw[R_ZETAS] ; p->zdn0 = raw[R_ZDN] ; p->zpn0 = raw[R_ZPN] ; p->zsn0 = raw[R_ZSN] ;
    /* . FillBetaUspd. */
    p->beta0 = ( Real * ) calloc ( norbitals, sizeof ( Real ) ) ;
    p->uspd0 = ( Real * ) calloc ( norbitals, sizeof ( Real ) ) ;
    p->beta0[0] = p->betas0 ; p->uspd0[0] = p->uss0 ;
    for ( i = 1 ; i < norbitals && i < 4 ; i++ ) { p->beta0[i] = p->betap0 ; p->uspd0[i] = p->upp0 ; }
    /* . FillFN123 / FillPDDG. */
    if ( nGaussians > 0 )
    {
        p->nam1pm3g = nGaussians ;
        p->fn10 = ( Real * ) calloc ( nGaussians, sizeof ( Real ) ) ;
        p->fn20 = ( Real * ) calloc ( nGaussians, sizeof ( Real ) ) ;
        p->fn30 = ( Real * ) calloc ( nGaussians, sizeof ( Real ) ) ;
        for ( i = 0 ; i < nGaussians ; i++ ) { p->fn10[i] = gaussians[3*i] ; p->fn20[i] = gaussians[3*i+1] ; p->fn30[i] = gaussians[3*i+2] ; }
    }
    if ( nPDDG > 0 )
    {
        p->npddg = nPDDG ;
        p->pddgc0 = ( Real * ) calloc ( nPDDG, sizeof ( Real ) ) ;
        p->pddge0 = ( Real * ) calloc ( nPDDG, sizeof ( Real ) ) ;
        for ( i = 0 ; i < nPDDG ; i++ ) { p->pddgc0[i] = pddg[2*i] ; p->pddge0[i] = pddg[2*i+1] ; }
    }
    /* . FillDiatomic (pMolecule.MNDOParameters.pyx:259-276): rows (partner atomic number, x, a), indexed by the
         partner's atomic number up to the largest one. */
    if ( nDiatomic > 0 )
    {
        int maxZ = 0 ;
        for ( i = 0 ; i < nDiatomic ; i++ ) if ( ( int ) diatomic[3*i] > maxZ ) maxZ = ( int ) diatomic[3*i] ;
        p->QDIATOMIC      = True ;
        p->ndiatomic      = maxZ + 1 ;
        p->QDIATOMICFLAGS = ( Boolean * ) calloc ( p->ndiatomic, sizeof ( Boolean ) ) ;
        p->diatomica0     = ( Real    * ) calloc ( p->ndiatomic, sizeof ( Real    ) ) ;
        p->diatomicx0     = ( Real    * ) calloc ( p->ndiatomic, sizeof ( Real    ) ) ;
        for ( i = 0 ; i < nDiatomic ; i++ )
        {
            int j = ( int ) diatomic[3*i] ;
            p->QDIATOMICFLAGS[j] = True ;
            p->diatomicx0[j] = diatomic[3*i+1] ;
            p->diatomica0[j] = diatomic[3*i+2] ;
        }
    }
    /* . ToAtomicUnits. */
    p->ad    = p->ad0 ;
    p->alp   = p->alp0 * BOHRS_TO_ANGSTROMS ;
    p->am    = p->am0 ;
    p->aq    = p->aq0 ;
    p->betad = p->betad0 / HARTREES_TO_EV ;
    p->betap = p->betap0 / HARTREES_TO_EV ;
    p->betas = p->betas0 / HARTREES_TO_EV ;
    p->dd    = p->dd0 ;
    p->eheat = p->eheat0 / HARTREES_TO_KCAL ;
    p->eisol = p->eisol0 / HARTREES_TO_EV ;
    p->f0sd  = p->f0sd0  / HARTREES_TO_EV ;
    p->gphot = p->gphot0 ;
    p->gpp   = p->gpp0   / HARTREES_TO_EV ;
    p->gp2   = p->gp20   / HARTREES_TO_EV ;
    p->gsp   = p->gsp0   / HARTREES_TO_EV ;
    p->gss   = p->gss0   / HARTREES_TO_EV ;
    p->g2sd  = p->g2sd0  / HARTREES_TO_EV ;
    p->hsp   = p->hsp0   / HARTREES_TO_EV ;
    p->pcore = p->pcore0 ;
    p->qq    = p->qq0 ;
    p->udd   = p->udd0   / HARTREES_TO_EV ;
    p->upp   = p->upp0   / HARTREES_TO_EV ;
    p->uss   = p->uss0   / HARTREES_TO_EV ;
    p->zcore = p->zcore0 ;
    p->zetad = p->zetad0 ; p->zetap = p->zetap0 ; p->zetas = p->zetas0 ;
    p->zdn   = p->zdn0   ; p->zpn   = p->zpn0   ; p->zsn   = p->zsn0   ;
    p->beta = ( Real * ) calloc ( norbitals, sizeof ( Real ) ) ;
    p->uspd = ( Real * ) calloc ( norbitals, sizeof ( Real ) ) ;
    for ( i = 0 ; i < norbitals ; i++ ) { p->beta[i] = p->beta0[i] / HARTREES_TO_EV ; p->uspd[i] = p->uspd0[i] / HARTREES_TO_EV ; }
    if ( p->nam1pm3g > 0 )
    {
        p->fn1 = ( Real * ) calloc ( p->nam1pm3g, sizeof ( Real ) ) ;
        p->fn2 = ( Real * ) calloc ( p->nam1pm3g, sizeof ( Real ) ) ;
        p->fn3 = ( Real * ) calloc ( p->nam1pm3g, sizeof ( Real ) ) ;
        for ( i = 0 ; i < p->nam1pm3g ; i++ )
        {
            p->fn1[i] = p->fn10[i] / ( BOHRS_TO_ANGSTROMS * HARTREES_TO_EV ) ;
            p->fn2[i] = p->fn20[i] * BOHRS_TO_ANGSTROMS * BOHRS_TO_ANGSTROMS ;
            p->fn3[i] = p->fn30[i] / BOHRS_TO_ANGSTROMS ;
        }
    }
    if ( p->npddg > 0 )
    {
        p->pddgc = ( Real * ) calloc ( p->npddg, sizeof ( Real ) ) ;
        p->pddge = ( Real * ) calloc ( p->npddg, sizeof ( Real ) ) ;
        for ( i = 0 ; i < p->npddg ; i++ ) { p->pddgc[i] = p->pddgc0[i] / HARTREES_TO_EV ; p->pddge[i] = p->pddge0[i] / BOHRS_TO_ANGSTROMS ; }
    }
    if ( p->ndiatomic > 0 )   /* . pMolecule.MNDOParameters.pyx:358-363 */
    {
        p->diatomica = ( Real * ) calloc ( p->ndiatomic, sizeof ( Real ) ) ;
        p->diatomicx = ( Real * ) calloc ( p->ndiatomic, sizeof ( Real ) ) ;
        for ( i = 0 ; i < p->ndiatomic ; i++ ) { p->diatomica[i] = p->diatomica0[i] * BOHRS_TO_ANGSTROMS ; p->diatomicx[i] = p->diatomicx0[i] ; }
    }
    MNDOParameters_CalculateOneCenterTEIs ( p ) ;
    return p ;
}

/* . Orbital basis, pMolecule.GaussianBasis.pyx:96-122 then QCParameters.pyx:131-140. */
static GaussianBasis *MakeBasis ( const int atomicNumber, const int nShells, const int *shellTypes, const int *nPrimitives,
                                  const double *exponents, const double *coefficients, const MNDOParameters *p )
{
    int i, s ;
    GaussianBasis *b = GaussianBasis_Allocate ( nShells ) ;
    b->atomicNumber = atomicNumber ;
    b->QSPHERICAL = True ;
    b->QNORMALIZEDPRIMITIVES = True ;
    for ( s = 0 ; s < nShells ; s++ )
    {
        GaussianBasis_AllocateShell ( b, s, nPrimitives[s], shellTypes[s] ) ;
        for ( i = 0 ; i < nPrimitives[s] ; i++ )
        {
            b->shells[s].primitives[i].exponent  = b->shells[s].primitives[i].exponent0 = exponents[s*MAXPRIM+i] ;
            b->shells[s].primitives[i].coefficients[0] = b->shells[s].primitives[i].coefficients0[0] = coefficients[s*MAXPRIM+i] ;
        }
    }
    b->type = GaussianBasisType_Orbital ;
    GaussianBasis_UnnormalizePrimitives ( b ) ;
    GaussianBasis_Normalize ( b ) ;
    GaussianBasis_ScaleExponents ( b, p->zetas, p->zetap, p->zetad ) ;
    return b ;
}

void *ref_hamiltonian_create ( const int nElements, const int *atomicNumbers, const int *norbitals, const double *raw,
                               const int *nGaussians, const double *gaussians, const int *nPDDG, const double *pddg,
                               const int *nShells, const int *shellTypes, const int *nPrimitives,
                               const double *exponents, const double *coefficients, const int *nDiatomic, const double *diatomic )
{
    int e ;
    RefHamiltonian *h = ( RefHamiltonian * ) calloc ( 1, sizeof ( RefHamiltonian ) ) ;
    h->nElements     = nElements ;
    h->atomicNumbers = ( int * ) calloc ( nElements, sizeof ( int ) ) ;
    h->parameters    = QCParameters_Allocate ( nElements ) ;
    for ( e = 0 ; e < nElements ; e++ )
    {
        MNDOParameters *p ;
        h->atomicNumbers[e] = atomicNumbers[e] ;
        p = MakeElement ( atomicNumbers[e], norbitals[e], raw + e*NRAW, nGaussians[e], gaussians + e*MAXGAUSS*3, nPDDG[e], pddg + e*MAXPDDG*2,
                          nDiatomic[e], diatomic + e*MAXDIATOMIC*3 ) ;
        h->parameters->centers[e].atomicNumber   = atomicNumbers[e] ;
        h->parameters->centers[e].mndoparameters = p ;
        h->parameters->centers[e].orbitalbasis   = MakeBasis ( atomicNumbers[e], nShells[e], shellTypes + 2*e, nPrimitives + 2*e,
                                                               exponents + e*2*MAXPRIM, coefficients + e*2*MAXPRIM, p ) ;
    }
    return h ;
}

/* . Derived per-element quantities for checking the host-side parameter processing.
!  . out: po[9], ddp[6], dd, qq, am, ad, aq, alp, zcore, eheat, eisol, gss, gsp, gpp, gp2, hsp, hpp, beta[4], uspd[4],
!  .      fn1/fn2/fn3[4 each], pddgc/pddge[4 each], one-centre TEI values[16], c2o[4x4] of the basis (row-major, zero padded). */
int ref_element_derived ( void *vh, const int e, double *out )
{
    RefHamiltonian *h = ( RefHamiltonian * ) vh ;
    MNDOParameters *p ;
    GaussianBasis  *b ;
    int i, j, n = 0 ;
    if ( ( h == NULL ) || ( e < 0 ) || ( e >= h->nElements ) ) return 4 ;
    p = h->parameters->centers[e].mndoparameters ;
    b = h->parameters->centers[e].orbitalbasis ;
    for ( i = 0 ; i < 9 ; i++ ) out[n++] = p->po[i] ;
    for ( i = 0 ; i < 6 ; i++ ) out[n++] = p->ddp[i] ;
    out[n++] = p->dd ; out[n++] = p->qq ; out[n++] = p->am ; out[n++] = p->ad ; out[n++] = p->aq ; out[n++] = p->alp ;
    out[n++] = p->zcore ; out[n++] = p->eheat ; out[n++] = p->eisol ;
    out[n++] = p->gss ; out[n++] = p->gsp ; out[n++] = p->gpp ; out[n++] = p->gp2 ; out[n++] = p->hsp ; out[n++] = p->hpp ;
    for ( i = 0 ; i < 4 ; i++ ) out[n++] = ( i < p->norbitals ) ? p->beta[i] : 0.0 ;
    for ( i = 0 ; i < 4 ; i++ ) out[n++] = ( i < p->norbitals ) ? p->uspd[i] : 0.0 ;
    for ( i = 0 ; i < 4 ; i++ ) out[n++] = ( i < p->nam1pm3g ) ? p->fn1[i] : 0.0 ;
    for ( i = 0 ; i < 4 ; i++ ) out[n++] = ( i < p->nam1pm3g ) ? p->fn2[i] : 0.0 ;
    for ( i = 0 ; i < 4 ; i++ ) out[n++] = ( i < p->nam1pm3g ) ? p->fn3[i] : 0.0 ;
    for ( i = 0 ; i < 4 ; i++ ) out[n++] = ( i < p->npddg ) ? p->pddgc[i] : 0.0 ;
    for ( i = 0 ; i < 4 ; i++ ) out[n++] = ( i < p->npddg ) ? p->pddge[i] : 0.0 ;
    for ( i = 0 ; i < 16 ; i++ ) out[n++] = ( i < p->nocteis ) ? p->octeivalues[i] : 0.0 ;
    for ( i = 0 ; i < 4 ; i++ )
    {
        for ( j = 0 ; j < 4 ; j++ ) out[n++] = ( ( i < b->c2o->length0 ) && ( j < b->c2o->length1 ) ) ? Real2DArray_Item ( b->c2o, i, j ) : 0.0 ;
    }
    return 0 ;
}

/* . Contracted coefficients (ccbf, unnormalized-primitive convention) and exponents per shell for checking. */
int ref_element_basis ( void *vh, const int e, double *exponents, double *ccbf )
{
    RefHamiltonian *h = ( RefHamiltonian * ) vh ;
    GaussianBasis  *b ;
    int i, s ;
    if ( ( h == NULL ) || ( e < 0 ) || ( e >= h->nElements ) ) return 4 ;
    b = h->parameters->centers[e].orbitalbasis ;
    for ( s = 0 ; s < b->nshells ; s++ )
    {
        for ( i = 0 ; i < b->shells[s].nprimitives ; i++ )
        {
            exponents[s*MAXPRIM+i] = b->shells[s].primitives[i].exponent ;
            ccbf     [s*MAXPRIM+i] = b->shells[s].primitives[i].ccbf[0] ;
        }
    }
    return 0 ;
}

/* . System set-up: QC atom container (QCAtomContainer.pyx:218-278), model and state (QCModelMNDO.pyx:623-672).
!  . alphaCharge / betaCharge as QCModel.CrossCheckModelAndState forms them (pMolecule.QCModel.pyx:99-118); the
!  . state as QCModelMNDOState_Setup (QCModelMNDOState.c) with the model's occupancy options; nFractional: the
!  . numbers of fractionally occupied HOOs / LUOs (restricted), then alpha HOOs / LUOs and beta HOOs / LUOs. */
static RefSystem *MakeSystem ( RefHamiltonian *h, const int nAtoms, const int *elementIndex, const int withQCMM,
                               const double densityTolerance, const int maximumSCFCycles, const int history,
                               const double diisOnset, const double energyTolerance, const int useRCA,
                               const int openShell, const double alphaCharge, const double betaCharge, const int isSpinRestricted,
                               const int occupancyType, const int *nFractional, const double fermiBroadening, const int charge )
{
    RefSystem *s ;
    QCAtomContainer *a ;
    int i, nElectrons ;
    if ( ( h == NULL ) || ( nAtoms <= 0 ) ) return NULL ;
    s = ( RefSystem * ) calloc ( 1, sizeof ( RefSystem ) ) ;
    s->hamiltonian = h ;
    s->nAtoms = nAtoms ;
    a = QCAtomContainer_Allocate ( nAtoms ) ;
    for ( i = 0 ; i < nAtoms ; i++ )
    {
        int c = elementIndex[i] ;
        GaussianBasis  *b = h->parameters->centers[c].orbitalbasis ;
        MNDOParameters *p = h->parameters->centers[c].mndoparameters ;
        a->data[i].index        = i ;
        a->data[i].atomicNumber = h->atomicNumbers[c] ;
        a->data[i].center       = c ;
        a->data[i].ostart       = a->nobasis  ;
        a->data[i].nobasis      = b->nbasis   ;
        a->data[i].ostartw      = a->nobasisw ;
        a->data[i].nobasisw     = b->nbasisw  ;
        a->nobasis  += b->nbasis  ;
        a->nobasisw += b->nbasisw ;
        a->nuclearCharge  += ( int ) lround ( p->zcore ) ;
        a->energybaseline += ( p->eheat - p->eisol ) ;
    }
    s->qcAtoms = a ;
    nElectrons = a->nuclearCharge - charge ;
    s->model = QCModelMNDO_Allocate ( ) ;
    if ( openShell )
    {
        s->model->isSpinRestricted = isSpinRestricted ? True : False ;
        s->model->occupancyType    = ( QCOnePDMOccupancyType ) occupancyType ;
        s->model->fermiBroadening  = fermiBroadening ;
        s->state = QCModelMNDOState_Setup ( a, h->parameters, alphaCharge, betaCharge, s->model->occupancyType, s->model->isSpinRestricted,
                                            nFractional[0], nFractional[1], nFractional[2], nFractional[3], nFractional[4], nFractional[5],
                                            s->model->fermiBroadening ) ;
    }
    else
        s->state = QCModelMNDOState_Setup ( a, h->parameters, 0.5 * nElectrons, 0.5 * nElectrons, s->model->occupancyType, True,
                                            0, 0, 0, 0, 0, 0, s->model->fermiBroadening ) ;
    s->converger = DIISSCFConverger_Allocate ( ) ;
    s->converger->densityTolerance = densityTolerance ;
    s->converger->maximumSCFCycles = maximumSCFCycles ;
    s->converger->ndiis            = history ;
    s->converger->diisonset        = diisOnset ;
    s->converger->energytolerance  = energyTolerance ;
    s->converger->QUSERCA          = ( useRCA ? True : False ) ;
    s->coordinates3 = Coordinates3_Allocate ( nAtoms ) ;
    s->gradients3   = Coordinates3_Allocate ( nAtoms ) ;
    if ( withQCMM ) s->qcmm = QCMMInteractionState_Allocate ( nAtoms, False, NULL ) ;
    return s ;
}

void *ref_system_create ( void *vh, const int nAtoms, const int *elementIndex, const int charge, const int withQCMM,
                          const double densityTolerance, const int maximumSCFCycles, const int history,
                          const double diisOnset, const double energyTolerance, const int useRCA )
{
    return MakeSystem ( ( RefHamiltonian * ) vh, nAtoms, elementIndex, withQCMM, densityTolerance, maximumSCFCycles, history,
                        diisOnset, energyTolerance, useRCA, 0, 0.0, 0.0, 1, 0, NULL, 0.0, charge ) ;
}

/* . Open-shell and fractional-occupancy states (QCModelMNDO keywords isSpinRestricted, occupancyType (0 cardinal,
!  . 1 fixed fractional, 2 variable fractional), numberFractional*, fermiBroadening). */
void *ref_system_create_open ( void *vh, const int nAtoms, const int *elementIndex, const double alphaCharge, const double betaCharge,
                               const int isSpinRestricted, const int occupancyType, const int *nFractional, const double fermiBroadening,
                               const int withQCMM, const double densityTolerance, const int maximumSCFCycles, const int history,
                               const double diisOnset, const double energyTolerance, const int useRCA )
{
    return MakeSystem ( ( RefHamiltonian * ) vh, nAtoms, elementIndex, withQCMM, densityTolerance, maximumSCFCycles, history,
                        diisOnset, energyTolerance, useRCA, 1, alphaCharge, betaCharge, isSpinRestricted, occupancyType,
                        nFractional, fermiBroadening, 0 ) ;
}

/* . The state's densities (packed lower triangles): restricted, the total density in p (q untouched); unrestricted,
!  . alpha in p and beta in q.  Returns 1 for unrestricted states. */
int ref_system_get_densities ( void *vs, double *p, double *q )
{
    RefSystem *s = ( RefSystem * ) vs ;
    if ( s == NULL ) return -1 ;
    memcpy ( p, s->state->densityp->density->data, sizeof ( double ) * s->state->densityp->density->size ) ;
    if ( s->state->densityq == NULL ) return 0 ;
    if ( q != NULL ) memcpy ( q, s->state->densityq->density->data, sizeof ( double ) * s->state->densityq->density->size ) ;
    return 1 ;
}

int ref_system_nbasis ( void *vs ) { RefSystem *s = ( RefSystem * ) vs ; return ( s == NULL ) ? -1 : s->qcAtoms->nobasis ; }

static void SetCoordinates ( RefSystem *s, const double *xyz )
{
    int i ;
    for ( i = 0 ; i < s->nAtoms ; i++ ) Coordinates3_SetRow ( s->coordinates3, i, xyz[3*i], xyz[3*i+1], xyz[3*i+2] ) ;
}

/* . The density currently held by the state (packed lower triangle, total density). */
int ref_system_get_density ( void *vs, double *density )
{
    RefSystem *s = ( RefSystem * ) vs ;
    if ( s == NULL ) return 4 ;
    memcpy ( density, s->state->densityp->density->data, sizeof ( double ) * s->state->densityp->density->size ) ;
    return 0 ;
}

int ref_system_set_density ( void *vs, const double *density )
{
    RefSystem *s = ( RefSystem * ) vs ;
    if ( s == NULL ) return 4 ;
    memcpy ( s->state->densityp->density->data, density, sizeof ( double ) * s->state->densityp->density->size ) ;
    s->state->densityp->isValid = True ;
    return 0 ;
}

/* . One energy (and optionally gradient) evaluation: System.Energy for the QC part, QCModel.pyx:146-185.
!  . xyz in Angstroms; qcmmPotentials in atomic units (ignored unless the system was made with QC/MM).
!  . energies: [eelectronic (QCModel.Energy sum incl. QC/MM), eelectronic (state), enuclear, energybaseline, eqcmm, eocc, eoei, etei].
!  . gradients: kJ/mol/A.  oneElectron (packed, nullable) receives the one-electron matrix.
!  . Returns 0 on convergence, 1 otherwise. */
int ref_system_energy ( void *vs, const double *xyz, const double *qcmmPotentials, const int doGradients,
                        double *energies, double *gradients, double *charges, double *oneElectron, int *ncycles )
{
    RefSystem *s = ( RefSystem * ) vs ;
    DIISSCFConvergerState *cs ;
    Real eelectronic = 0.0 ;
    int i, converged ;
    if ( s == NULL ) return 4 ;
    SetCoordinates ( s, xyz ) ;
    if ( doGradients ) Coordinates3_Set ( s->gradients3, 0.0 ) ;
    if ( s->qcmm != NULL )
    {
        for ( i = 0 ; i < s->nAtoms ; i++ ) Real1DArray_Item ( s->qcmm->qcmmPotentials, i ) = ( qcmmPotentials == NULL ) ? 0.0 : qcmmPotentials[i] ;
    }
    QCModelMNDOState_Initialize ( s->state, s->coordinates3, s->qcmm, ( doGradients ? s->gradients3 : NULL ) ) ;
    QCModelMNDO_Integrals ( s->model, s->state ) ;
    if ( oneElectron != NULL ) memcpy ( oneElectron, s->state->oneelectronmatrix->data, sizeof ( double ) * s->state->oneelectronmatrix->size ) ;
    cs = DIISSCFConvergerState_SetUp ( s->converger->QUSERCA, s->converger->ndiis, s->state->densityp, s->state->densityq, NULL, NULL ) ;
    while ( DIISSCFConverger_Continue ( s->converger, cs ) )
    {
        QCModelMNDO_Fock           ( s->model, s->state, &eelectronic ) ;
        QCModelMNDO_QCMMFockLowdin ( s->model, s->state, &eelectronic ) ;
        if ( DIISSCFConverger_Converged ( s->converger, cs ) != True )
        {
            DIISSCFConverger_IterateWithoutDensities ( s->converger, cs, eelectronic ) ;
            DIISSCFConverger_MakeDensities           ( s->converger, cs ) ;
        }
    }
    converged = ( cs->isConverged == True ) ;
    if ( ncycles != NULL ) (*ncycles) = cs->iteration ;
    DIISSCFConvergerState_Deallocate ( &cs ) ;
    energies[0] = eelectronic ;
    energies[1] = s->state->eelectronic ;
    energies[2] = s->state->enuclear ;
    energies[3] = s->qcAtoms->energybaseline ;
    energies[4] = s->state->eqcmm ;
    energies[5] = s->state->eocc ;
    energies[6] = s->state->eoei ;
    energies[7] = s->state->etei ;
    if ( ( charges != NULL ) && ( s->qcmm != NULL ) )
    {
        for ( i = 0 ; i < s->nAtoms ; i++ ) charges[i] = Real1DArray_Item ( s->qcmm->qcCharges, i ) ;
    }
    if ( doGradients && converged )
    {
        QCModelMNDO_Gradients ( s->model, s->state ) ;
        for ( i = 0 ; i < s->nAtoms ; i++ ) Coordinates3_GetRow ( s->gradients3, i, gradients[3*i], gradients[3*i+1], gradients[3*i+2] ) ;
    }
    QCModelMNDOState_Finalize ( s->state, s->model->keepOrbitalData ) ;
    return ( converged ? 0 : 1 ) ;
}

/* . Fock matrix and electronic energy for a given density, no SCF (QCModelMNDO_Fock + QCMMFockLowdin on one density). */
int ref_system_fock ( void *vs, const double *xyz, const double *qcmmPotentials, const double *density, double *fock, double *energies )
{
    RefSystem *s = ( RefSystem * ) vs ;
    Real eelectronic = 0.0 ;
    int i ;
    if ( s == NULL ) return 4 ;
    SetCoordinates ( s, xyz ) ;
    if ( s->qcmm != NULL )
    {
        for ( i = 0 ; i < s->nAtoms ; i++ ) Real1DArray_Item ( s->qcmm->qcmmPotentials, i ) = ( qcmmPotentials == NULL ) ? 0.0 : qcmmPotentials[i] ;
    }
    QCModelMNDOState_Initialize ( s->state, s->coordinates3, s->qcmm, NULL ) ;
    QCModelMNDO_Integrals ( s->model, s->state ) ;
    memcpy ( s->state->densityp->density->data, density, sizeof ( double ) * s->state->densityp->density->size ) ;
    QCModelMNDO_Fock           ( s->model, s->state, &eelectronic ) ;
    QCModelMNDO_QCMMFockLowdin ( s->model, s->state, &eelectronic ) ;
    memcpy ( fock, s->state->densityp->fock->data, sizeof ( double ) * s->state->densityp->fock->size ) ;
    energies[0] = eelectronic ;
    energies[1] = s->state->eelectronic ;
    energies[2] = s->state->enuclear ;
    QCModelMNDOState_Finalize ( s->state, s->model->keepOrbitalData ) ;
    return 0 ;
}

/* . Gradients (kJ/mol/A) for a given density, no SCF. */
int ref_system_gradients ( void *vs, const double *xyz, const double *density, double *gradients )
{
    RefSystem *s = ( RefSystem * ) vs ;
    int i ;
    if ( s == NULL ) return 4 ;
    SetCoordinates ( s, xyz ) ;
    Coordinates3_Set ( s->gradients3, 0.0 ) ;
    QCModelMNDOState_Initialize ( s->state, s->coordinates3, NULL, s->gradients3 ) ;
    QCModelMNDO_Integrals ( s->model, s->state ) ;
    memcpy ( s->state->densityp->density->data, density, sizeof ( double ) * s->state->densityp->density->size ) ;
    QCModelMNDO_Gradients ( s->model, s->state ) ;
    for ( i = 0 ; i < s->nAtoms ; i++ ) Coordinates3_GetRow ( s->gradients3, i, gradients[3*i], gradients[3*i+1], gradients[3*i+2] ) ;
    QCModelMNDOState_Finalize ( s->state, s->model->keepOrbitalData ) ;
    return 0 ;
}

void ref_system_free ( void *vs )
{
    RefSystem *s = ( RefSystem * ) vs ;
    if ( s == NULL ) return ;
    QCModelMNDOState_Deallocate ( &s->state ) ;
    QCModelMNDO_Deallocate ( &s->model ) ;
    DIISSCFConverger_Deallocate ( &s->converger ) ;
    QCAtomContainer_Deallocate ( &s->qcAtoms ) ;
    Coordinates3_Deallocate ( &s->coordinates3 ) ;
    Coordinates3_Deallocate ( &s->gradients3 ) ;
    if ( s->qcmm != NULL ) QCMMInteractionState_Deallocate ( &s->qcmm ) ;
    free ( s ) ;
}

/*----------------------------------------------------------------------------------------------------------------------------------
! . QC/MM electrostatics through the reference ABFS pair routines (PairwiseInteraction.c:542,612).
! . The spline knots (x = r^2 in A^2, y in atomic units) are supplied by the caller.
!---------------------------------------------------------------------------------------------------------------------------------*/
void *ref_abfs_create ( const double innerCutoff, const double outerCutoff, const int n, const double *x, const double *y )
{
    PairwiseInteractionABFS *p = PairwiseInteractionABFS_Allocate ( ) ;
    Real1DArray *rx = Real1DArray_Allocate ( n, NULL ), *ry = Real1DArray_Allocate ( n, NULL ) ;
    int i ;
    for ( i = 0 ; i < n ; i++ ) { Real1DArray_Item ( rx, i ) = x[i] ; Real1DArray_Item ( ry, i ) = y[i] ; }
    p->innerCutoff = innerCutoff ;
    p->outerCutoff = outerCutoff ;
    p->dampingCutoff = 0.0 ;
    CubicSpline_Deallocate ( &p->electrostaticSpline ) ;
    CubicSpline_MakeFromReal1DArrays ( &p->electrostaticSpline, &rx, &ry, 1, 0.0, 1, 0.0 ) ;
    return p ;
}

/* . Spline value and derivative d/d(r^2) at x (for checking the device evaluation). */
int ref_abfs_spline ( void *vp, const int n, const double *x, double *f, double *g )
{
    PairwiseInteractionABFS *p = ( PairwiseInteractionABFS * ) vp ;
    int i ;
    for ( i = 0 ; i < n ; i++ ) CubicSpline_Evaluate ( p->electrostaticSpline, x[i], &f[i], &g[i], NULL ) ;
    return 0 ;
}

/* . Potentials (a.u.) at QC atoms and gradients (kJ/mol/A) on QC and MM atoms.
!  . The pair list holds every (QC, MM) pair; the reference skips pairs beyond the outer cutoff itself. */
int ref_abfs_qcmm ( void *vp, void *vs, const double *qcxyz, const int nMM, const double *mmxyz, const double *mmCharges,
                    const double *qcCharges, double *potentials, double *qcGradients, double *mmGradients )
{
    /* . The pair list indexes MM atoms after the QC atoms, as system-wide atom indices do in pDynamo
       (PairList_FromIntegerPairArray drops pairs with equal indices). */
    PairwiseInteractionABFS *p = ( PairwiseInteractionABFS * ) vp ;
    RefSystem *s = ( RefSystem * ) vs ;
    int nq = s->nAtoms, nt = s->nAtoms + nMM ;
    Coordinates3 *crd1 = Coordinates3_Allocate ( nq ), *crd2 = Coordinates3_Allocate ( nt ) ;
    Coordinates3 *grd1 = Coordinates3_Allocate ( nq ), *grd2 = Coordinates3_Allocate ( nt ) ;
    Real1DArray *q = Real1DArray_Allocate ( nt, NULL ), *phi = Real1DArray_Allocate ( nq, NULL ), *qc = Real1DArray_Allocate ( nq, NULL ) ;
    Integer *indices = ( Integer * ) malloc ( sizeof ( Integer ) * 2 * ( size_t ) nq * nMM ) ;
    PairList *list ;
    int i, m, n = 0 ;
    Coordinates3_Set ( crd2, 0.0 ) ; Real1DArray_Set ( q, 0.0 ) ;
    for ( i = 0 ; i < nq ; i++ ) { Coordinates3_SetRow ( crd1, i, qcxyz[3*i], qcxyz[3*i+1], qcxyz[3*i+2] ) ; Real1DArray_Item ( qc, i ) = qcCharges[i] ; }
    for ( m = 0 ; m < nMM ; m++ ) { Coordinates3_SetRow ( crd2, nq + m, mmxyz[3*m], mmxyz[3*m+1], mmxyz[3*m+2] ) ; Real1DArray_Item ( q, nq + m ) = mmCharges[m] ; }
    for ( i = 0 ; i < nq ; i++ ) for ( m = 0 ; m < nMM ; m++ ) { indices[n++] = i ; indices[n++] = nq + m ; }
    list = PairList_FromIntegerPairArray ( False, nq * nMM, indices ) ;
    Real1DArray_Set ( phi, 0.0 ) ;
    Coordinates3_Set ( grd1, 0.0 ) ; Coordinates3_Set ( grd2, 0.0 ) ;
    PairwiseInteractionABFS_QCMMPotentials ( p, q, s->qcAtoms, list, 1.0, crd1, crd2, phi ) ;
    PairwiseInteractionABFS_QCMMGradients  ( p, q, s->qcAtoms, list, 1.0, crd1, crd2, qc, grd1, grd2 ) ;
    for ( i = 0 ; i < nq ; i++ ) { potentials[i] = Real1DArray_Item ( phi, i ) ; Coordinates3_GetRow ( grd1, i, qcGradients[3*i], qcGradients[3*i+1], qcGradients[3*i+2] ) ; }
    for ( m = 0 ; m < nMM ; m++ ) Coordinates3_GetRow ( grd2, nq + m, mmGradients[3*m], mmGradients[3*m+1], mmGradients[3*m+2] ) ;
    PairList_Deallocate ( &list ) ;
    free ( indices ) ;
    Coordinates3_Deallocate ( &crd1 ) ; Coordinates3_Deallocate ( &crd2 ) ;
    Coordinates3_Deallocate ( &grd1 ) ; Coordinates3_Deallocate ( &grd2 ) ;
    Real1DArray_Deallocate ( &q ) ; Real1DArray_Deallocate ( &phi ) ; Real1DArray_Deallocate ( &qc ) ;
    return 0 ;
}

/*----------------------------------------------------------------------------------------------------------------------------------
! . MM/MM electrostatic and LJ energies and QC/MM LJ energies of NBModelABFS (no symmetry), through the reference's
! . pair-list generator and PairwiseInteractionABFS_MMMMEnergy (PairwiseInteraction.c:292), analytic form.
! . flags per atom: bit 0 active MM atom (mmSelection), bit 1 QC atom with LJ interactions (qcpSelection),
! . bit 2 fixed.  Exclusions and 1-4 interactions as (i, j) pairs.  LJ types with epsilon (kJ/mol) and sigma (A)
! . turned into tables by the OPLS (opls != 0) or AMBER rule; 1-4 LJ from their own epsilon and sigma.
! . energies (kJ/mol): MM/MM Elect., MM/MM LJ, MM/MM 1-4 Elect., MM/MM 1-4 LJ, QC/MM LJ, QC/MM 1-4 LJ.
! . gradients (kJ/mol/A, nAtoms x 3) are overwritten.
!---------------------------------------------------------------------------------------------------------------------------------*/
static Selection *SelectFlag ( const int n, const int *flags, const int bit, const int want )
{
    Integer *ix = ( Integer * ) malloc ( sizeof ( Integer ) * ( size_t ) ( n > 0 ? n : 1 ) ) ;
    int i, k = 0 ;
    Selection *sel ;
    for ( i = 0 ; i < n ; i++ ) if ( ( ( flags[i] >> bit ) & 1 ) == want ) ix[k++] = i ;
    sel = Selection_FromIntegerArray ( k, ix ) ;
    free ( ix ) ;
    return sel ;
}

static LJParameterContainer *MakeLJ ( const int nTypes, const double *epsilon, const double *sigma, const int opls )
{
    LJParameterContainer *lj = LJParameterContainer_Allocate ( nTypes ) ;
    int t ;
    for ( t = 0 ; t < nTypes ; t++ ) { lj->epsilon[t] = epsilon[t] ; lj->sigma[t] = sigma[t] ; }
    if ( opls ) LJParameterContainer_MakeTableOPLS ( lj ) ;
    else        LJParameterContainer_MakeTableAMBER ( lj ) ;
    return lj ;
}

int ref_mmmm_energy ( const int nAtoms, const double *xyz, const double *charges, const int *ljTypes, const int *flags,
                      const int nTypes, const double *epsilon, const double *sigma, const double *epsilon14, const double *sigma14,
                      const int opls, const int nExclusions, const int *exclusions, const int n14, const int *pairs14,
                      const double innerCutoff, const double outerCutoff, const double dampingCutoff, const double listCutoff,
                      const double dielectric, const double scale14, double *energies, double *gradients )
{
    Coordinates3 *crd = Coordinates3_Allocate ( nAtoms ), *grd = Coordinates3_Allocate ( nAtoms ) ;
    MMAtomContainer *mm = MMAtomContainer_Allocate ( nAtoms ) ;
    LJParameterContainer *lj = MakeLJ ( nTypes, epsilon, sigma, opls ), *lj14 = MakeLJ ( nTypes, epsilon14, sigma14, opls ) ;
    PairwiseInteractionABFS *p = PairwiseInteractionABFS_Allocate ( ) ;
    PairListGenerator *g = PairListGenerator_Allocate ( ) ;
    Selection *mmSel = SelectFlag ( nAtoms, flags, 0, 1 ), *qcpSel = SelectFlag ( nAtoms, flags, 1, 1 ), *freeSel = NULL ;
    PairList *excl = NULL, *i14 = NULL, *nbmmmm = NULL, *nbqcmmlj = NULL, *nbmmmm14 = NULL, *nbqcmmlj14 = NULL ;
    RegularGrid *grid = NULL ;
    RegularGridOccupancy *occupancy = NULL ;
    Real eScale = 1.0 / dielectric ;
    int i, nFixed = 0 ;
    for ( i = 0 ; i < 6 ; i++ ) energies[i] = 0.0 ;
    for ( i = 0 ; i < nAtoms ; i++ )
    {
        Coordinates3_SetRow ( crd, i, xyz[3*i], xyz[3*i+1], xyz[3*i+2] ) ;
        mm->data[i].QACTIVE  = ( flags[i] & 1 ) ? True : False ;
        mm->data[i].atomtype = 0 ;
        mm->data[i].ljtype   = ljTypes[i] ;
        mm->data[i].charge   = charges[i] ;
        if ( ( flags[i] >> 2 ) & 1 ) nFixed++ ;
    }
    Coordinates3_Set ( grd, 0.0 ) ;
    /* . pMolecule.NBModelABFS.pyx:79-82: the MM/MM interaction takes the model's cutoffs (analytic form). */
    p->innerCutoff = innerCutoff ; p->outerCutoff = outerCutoff ; p->dampingCutoff = dampingCutoff ; p->useAnalyticForm = True ;
    /* . pMolecule.NBModelABFS.pyx:62-69 and pCore.PairListGenerator.pyx:104. */
    g->cutoff = listCutoff ; g->cutoffCellSizeFactor = 0.5 ; g->minimumCellExtent = 2 ; g->minimumCellSize = 3.0 ;
    g->minimumExtentFactor = 1.5 ; g->minimumPoints = 500 ; g->sortIndices = False ; g->useGridByCell = True ;
    g->cellSize = g->cutoffCellSizeFactor * g->cutoff ;
    if ( nFixed > 0 ) freeSel = SelectFlag ( nAtoms, flags, 2, 0 ) ;
    excl = PairList_FromIntegerPairArray ( True, nExclusions, ( Integer * ) exclusions ) ;
    if ( n14 > 0 ) i14 = PairList_FromIntegerPairArray ( True, n14, ( Integer * ) pairs14 ) ;
    /* . NBModelABFSState.c:207-226: a grid when the generator chooses a grid search. */
    if ( PairListGenerator_DetermineMethod ( g, crd, NULL ) ) Coordinates3_MakeGridAndOccupancy ( crd, NULL, g->cellSize, &grid, &occupancy, NULL ) ;
    /* . NBModelABFS.c:1050-1100 (GenerateLists). */
    nbmmmm   = PairListGenerator_SelfPairListFromCoordinates3 ( g, crd, NULL, mmSel, freeSel, excl, grid, occupancy, NULL ) ;
    nbqcmmlj = PairListGenerator_CrossPairListFromSingleCoordinates3 ( g, crd, NULL, qcpSel, mmSel, freeSel, excl, False, grid, occupancy, NULL ) ;
    /* . GenerateLists14. */
    if ( i14 != NULL )
    {
        nbmmmm14   = SelfPairList_FromSelfPairList ( i14, mmSel, freeSel, False ) ;
        nbqcmmlj14 = SelfPairList_ToCrossPairList  ( i14, qcpSel, mmSel, freeSel, False, False, False, False ) ;
    }
    /* . NBModelABFS.c:228-330 (MMMMEnergy, QCMMEnergyLJ; their 1-4 and QC/MM LJ lists). */
    if ( nbmmmm     != NULL ) PairwiseInteractionABFS_MMMMEnergy ( p, mm, lj,   nbmmmm,     eScale,           1.0, crd, crd, &energies[0], &energies[1], grd, grd ) ;
    if ( nbmmmm14   != NULL ) PairwiseInteractionABFS_MMMMEnergy ( p, mm, lj14, nbmmmm14,   eScale * scale14, 1.0, crd, crd, &energies[2], &energies[3], grd, grd ) ;
    if ( nbqcmmlj   != NULL ) PairwiseInteractionABFS_MMMMEnergy ( p, mm, lj,   nbqcmmlj,   0.0,              1.0, crd, crd, NULL,         &energies[4], grd, grd ) ;
    if ( nbqcmmlj14 != NULL ) PairwiseInteractionABFS_MMMMEnergy ( p, mm, lj14, nbqcmmlj14, 0.0,              1.0, crd, crd, NULL,         &energies[5], grd, grd ) ;
    for ( i = 0 ; i < nAtoms ; i++ ) Coordinates3_GetRow ( grd, i, gradients[3*i], gradients[3*i+1], gradients[3*i+2] ) ;
    PairList_Deallocate ( &nbmmmm ) ; PairList_Deallocate ( &nbqcmmlj ) ; PairList_Deallocate ( &nbmmmm14 ) ; PairList_Deallocate ( &nbqcmmlj14 ) ;
    PairList_Deallocate ( &excl ) ; PairList_Deallocate ( &i14 ) ;
    RegularGrid_Deallocate ( &grid ) ; RegularGridOccupancy_Deallocate ( &occupancy ) ;
    Selection_Deallocate ( &mmSel ) ; Selection_Deallocate ( &qcpSel ) ; Selection_Deallocate ( &freeSel ) ;
    PairListGenerator_Deallocate ( &g ) ; PairwiseInteractionABFS_Deallocate ( &p ) ;
    LJParameterContainer_Deallocate ( &lj ) ; LJParameterContainer_Deallocate ( &lj14 ) ; MMAtomContainer_Deallocate ( &mm ) ;
    Coordinates3_Deallocate ( &crd ) ; Coordinates3_Deallocate ( &grd ) ;
    return 0 ;
}

/*----------------------------------------------------------------------------------------------------------------------------------
! . Properties of the last energy's density: the dipole moment (Debye, about the origin; QCModelMNDO_DipoleMoment) and the
! . Mayer bond orders with the charges, free and total valences QCModelMNDO_MayerBondOrders gives (QCModelMNDO.c).
! . bondOrders: nAtoms x nAtoms (full).
!---------------------------------------------------------------------------------------------------------------------------------*/
int ref_system_properties ( void *vs, double *dipole, double *bondOrders, double *charges, double *freeValence, double *totalValence )
{
    RefSystem *s = ( RefSystem * ) vs ;
    int i, j, n ;
    Vector3 *d ;
    SymmetricMatrix *b ;
    Real1DArray *c, *f, *t ;
    if ( s == NULL ) return 4 ;
    n = s->nAtoms ;
    d = QCModelMNDO_DipoleMoment ( s->model, s->state, s->coordinates3, NULL ) ;
    for ( i = 0 ; i < 3 ; i++ ) dipole[i] = Vector3_Item ( d, i ) ;
    Vector3_Deallocate ( &d ) ;
    b = SymmetricMatrix_Allocate ( n ) ;
    c = Real1DArray_Allocate ( n, NULL ) ; f = Real1DArray_Allocate ( n, NULL ) ; t = Real1DArray_Allocate ( n, NULL ) ;
    QCModelMNDO_MayerBondOrders ( s->model, s->state, b, c, f, t ) ;
    for ( i = 0 ; i < n ; i++ )
    {
        for ( j = 0 ; j < n ; j++ ) bondOrders[i*n+j] = SymmetricMatrix_Get_Component ( b, i, j ) ;
        charges[i] = Real1DArray_Item ( c, i ) ; freeValence[i] = Real1DArray_Item ( f, i ) ; totalValence[i] = Real1DArray_Item ( t, i ) ;
    }
    SymmetricMatrix_Deallocate ( &b ) ;
    Real1DArray_Deallocate ( &c ) ; Real1DArray_Deallocate ( &f ) ; Real1DArray_Deallocate ( &t ) ;
    return 0 ;
}
