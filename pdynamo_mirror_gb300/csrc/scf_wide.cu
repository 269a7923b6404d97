// scf_wide.cu - the SCF kernels of scf.cu compiled for 512 threads per CTA and one CTA per SM (namespace
// scf_w), FP64 density steps only: one large molecule gets all sixteen warps (four per SM sub-partition) of
// its SM, where the 256-thread CTA leaves FP64 issue slots empty when it runs alone.
#define PDG_SCF_CTAS_PER_SM 1
#define PDG_SCF_NO_TENSOR 1
#define PDG_SCF_NS scf_w
#include "scf.cu"
