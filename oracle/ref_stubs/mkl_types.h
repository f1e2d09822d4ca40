// Stand-in for MKL's mkl_types.h (the reference's include/FE/Matrix.h
// includes it; nothing from it is used).  TEST INFRASTRUCTURE ONLY.
#ifndef REF_STUB_MKL_TYPES_H
#define REF_STUB_MKL_TYPES_H
#endif
