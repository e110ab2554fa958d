// ORACLE — test infrastructure only.
// Abort stubs for the LAPACK symbols referenced by the reference's generic
// matrix class (librarySources/matVecClasses/matvec2.cpp: dsyev/dgeev/zgeev/
// zgesv/zgemv/dpotrf/dpotri/dsteqr/spotrf/ssygst/cheev).  None of them is
// reachable from the NoQuad Hv path or the Lanczos driver; no LAPACK library
// exists in this image, so linking the reference needs these definitions.
#include <cstdio>
#include <cstdlib>
#define BSL_ORACLE_STUB(name) \
  extern "C" void name() { std::fprintf(stderr, "oracle: LAPACK " #name " is not available\n"); std::abort(); }
BSL_ORACLE_STUB(cheev_)
BSL_ORACLE_STUB(dgeev_)
BSL_ORACLE_STUB(dpotrf_)
BSL_ORACLE_STUB(dpotri_)
BSL_ORACLE_STUB(dsteqr_)
BSL_ORACLE_STUB(dsyev_)
BSL_ORACLE_STUB(spotrf_)
BSL_ORACLE_STUB(ssygst_)
BSL_ORACLE_STUB(zgeev_)
BSL_ORACLE_STUB(zgemv_)
BSL_ORACLE_STUB(zgesv_)
