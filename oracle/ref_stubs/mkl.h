// Stand-in for mkl.h, which the reference's NSE_MGLevel4 sources include
// without using anything from it on the harness's path.  TEST
// INFRASTRUCTURE ONLY.
#ifndef REF_STUB_MKL_H
#define REF_STUB_MKL_H
#endif
