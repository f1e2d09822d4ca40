// ref_hybrid_mapper.h — the cell colouring source of the reference's
// colour-parallel build, for the hybrid harness.  TEST INFRASTRUCTURE ONLY.
//
// Force-included (g++ -include) into every translation unit of
// oracle/_ref/libref_hybrid.so, which compiles the reference with -D_HYBRID
// instead of -D_SEQ.  In that build the TNSE_MGLevel4 constructor reads the
// cell colouring from its TParFEMapper3D argument (parMapper_P,
// src/FE/NSE_MGLevel4.C:315-324), a parameter the constructor has only in
// MPI builds (:126-128).  The build defines parMapper_P as a call of
// ref_hybrid_mapper(), whose object answers the same getters with no
// colours; the harness sets the level's colouring itself after construction
// (ref_vanka_set_colours in ref_vanka.cpp).
#ifndef REF_HYBRID_MAPPER_H
#define REF_HYBRID_MAPPER_H

struct RefHybridMapper {
  int GetN_CIntCell() const { return 0; }
  int *GetptrCellColors() const { return nullptr; }
  int *GetCellReorder() const { return nullptr; }
  int GetMaxCellsPerColor() const { return 0; }
  int GetN_CPDOF() const { return 0; }
  int *GetptrPDOFColors() const { return nullptr; }
  int *GetPDOFReorder() const { return nullptr; }
};

RefHybridMapper *ref_hybrid_mapper();

#endif
