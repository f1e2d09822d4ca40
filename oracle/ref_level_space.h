// ref_level_space.h — a TFESpace3D filled from a level's arrays, and the
// structures of a level's matrices over it, shared by the reference
// harnesses (ref_vanka.cpp, ref_transfer.cpp).  TEST INFRASTRUCTURE ONLY.
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
#include <SquareStructure3D.h>
#include <Structure3D.h>

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

// The structures of a level's matrices over LevelSpace objects: A's square
// structure with its active bound and space, and the B / BT structure (a
// TStructure3D built from two spaces on different collections, for which its
// constructor returns at once, src/FE/Structure3D.C:43-46, then given the
// pattern and the level's spaces).
struct LevelSquareStructure : public TSquareStructure3D {
  LevelSquareStructure(int n, int active, int nnz, int *col, int *rowptr, TFESpace3D *space)
      : TSquareStructure3D(n, nnz, col, rowptr) {
    ActiveBound = active;
    FESpace = space;
  }
};

struct LevelStructure : public TStructure3D {
  LevelStructure(TFESpace3D *other_a, TFESpace3D *other_b, TFESpace3D *test, TFESpace3D *ansatz,
                 int rows, int cols, int nnz, int *col, int *rowptr)
      : TStructure3D(other_a, other_b) {
    N_Rows = rows;
    N_Columns = cols;
    N_Entries = nnz;
    KCol = col;
    RowPtr = rowptr;
    HangingN_Entries = 0;
    HangingKCol = nullptr;
    HangingRowPtr = nullptr;
    TestSpace3D = test;
    AnsatzSpace3D = ansatz;
    TestSpace2D = nullptr;
    AnsatzSpace2D = nullptr;
  }
};

#endif
