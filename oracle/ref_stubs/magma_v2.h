// Stand-in for MAGMA's magma_v2.h: the three type names the reference's
// include/FE/Magma_Solver.h declares its members with.  The reference
// harness never creates a Magma_Solver (only CUDA builds of NSE_MGLevel4.C
// do).  TEST INFRASTRUCTURE ONLY.
#ifndef REF_STUB_MAGMA_V2_H
#define REF_STUB_MAGMA_V2_H
typedef int magma_int_t;
typedef void *magma_queue_t;
typedef double *magmaDouble_ptr;
#endif
