// ref_level_space.h — a TFESpace3D filled from a level's arrays, shared by
// the reference harnesses (ref_vanka.cpp, ref_transfer.cpp).  TEST
// INFRASTRUCTURE ONLY.
//
// The space's DOF maps (GlobalNumbers, BeginIndex), DOF count, active /
// hanging / Dirichlet bounds and per-cell element ids (AllElements, which
// TFESpace3D::GetFE3D returns before it would look at a cell,
// src/FE/FESpace3D.C:412-422) are set directly; there are no hanging nodes.
// The name strings come from TFESpace::InitData (strdup, src/FE/FESpace.C:24-27)
// and are freed by release_names(); no reference destructor runs.
#ifndef REF_LEVEL_SPACE_H
#define REF_LEVEL_SPACE_H

#include <cstdlib>

#include <Collection.h>
#include <FESpace3D.h>

struct LevelSpace : public TFESpace3D {
  LevelSpace(TCollection *coll, int n_dof, int active, int n_dirichlet, int *global, int *begin,
             FE3D *all)
      : TFESpace3D(coll, (char *)"harness", (char *)"harness") {
    N_DegreesOfFreedom = n_dof;
    GlobalNumbers = global;
    BeginIndex = begin;
    ActiveBound = active;
    HangingBound = active;
    DirichletBound = n_dof;
    InnerBound = active;
    N_Inner = active;
    N_Dirichlet = n_dirichlet;
    N_ActiveDegrees = active;
    N_SlaveDegrees = 0;
    AllElements = all;
  }
  void release_names() {
    std::free(Name);
    std::free(Description);
  }
};

#endif
