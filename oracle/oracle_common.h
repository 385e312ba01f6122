/*
 * oracle_common.h -- shared data model of the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  The oracle is a CPU FP64 restatement of the
 * reference (Fortran) algorithms of the afivo-streamer hot path, used by
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
 * checker.  The product (afivo-streamer_gb300/) never links or calls it.
 *
 * Data layout mirrors the reference's per-box arrays
 * (afivo/src/m_af_types.f90:302-303): cc[id-1][iv-1][(nc+2)^D], i fastest;
 * fc[id-1][ivf-1][dim][(nc+1)^D].
 *
 * Build with -ffp-contract=off: every expression follows the reference's
 * left-to-right evaluation order with no fused multiply-add, so that the
 * GPU FP64 path (built with --fmad=false) can be compared bit for bit.
 */
#ifndef ORACLE_COMMON_H
#define ORACLE_COMMON_H

#include <cstddef>
#include <cstdint>
#include <map>
#include <vector>

#include <memory>

#include "../include/afivo_gpu.h"
#include "../afivo-streamer_gb300/csrc/afg_lsf.h"

namespace orc {

struct Tree {
  int D = 2, nc = 16, coord = AFG_XYZ, n_boxes = 0, highest_lvl = 0;
  int n2 = 18, S = 324, NF = 289;  // nc+2, (nc+2)^D, (nc+1)^D
  int n_var = 0, n_var_face = 0;
  int cgs[3] = {0, 0, 0};
  std::vector<int> lvl, ix, parent, children, neighbors, nbmat;
  std::vector<double> r_min, dr;
  std::vector<std::vector<int>> ids, leaves, parents;  // [lvl-1]

  int nchild() const { return 1 << D; }
  int nnb() const { return 2 * D; }
  int nmat() const { return D == 2 ? 9 : 27; }
  int nb_of(int id, int nb) const { return neighbors[(size_t)(id - 1) * nnb() + nb]; }
  int child_of(int id, int c) const { return children[(size_t)(id - 1) * nchild() + c]; }
  int ix_of(int id, int d) const { return ix[(size_t)(id - 1) * D + d]; }
  double rmin_of(int id, int d) const { return r_min[(size_t)(id - 1) * D + d]; }
  double dr_of(int id, int d) const { return dr[(size_t)(id - 1) * D + d]; }
  /* neighbor_mat(dx,dy[,dz]), each in -1..1, first index fastest */
  int mat_of(int id, int dx, int dy, int dz) const {
    int k = (dx + 1) + 3 * (dy + 1) + (D == 3 ? 9 * (dz + 1) : 0);
    return nbmat[(size_t)(id - 1) * nmat() + k];
  }
  /* linear index of cell (i,j[,k]) inside a box array, 0..nc+1 each */
  inline int at(int i, int j, int k = 0) const { return i + n2 * (j + n2 * k); }
  inline double* var(double* cc, int id, int iv) const {
    return cc + ((size_t)(id - 1) * n_var + (iv - 1)) * S;
  }
  /* af_get_child_offset (m_af_types.f90:903-910) */
  int child_offset(int id, int d) const { return ((ix_of(id, d) - 1) & 1) * (nc / 2); }
};

struct GcSpec {
  int bc_type[6];
  double bc_val[6];
  int rb;
};

/* Electrode of a multigrid problem (tree%mg_i_lsf, mg%lsf): per box the
 * reference stores a distance matrix and a variable operator stencil
 * (store_lsf_distance_matrix, mg_box_lsf_stencil, m_af_multigrid.f90:
 * 977-1097, 1779-1853) with bc_correction = f * boundary value; here the
 * boxes that have them, with the per-cell arrays (cells i fastest). */
struct Lsf {
  afg_lsf::Electrode e{};
  int i_lsf = 0;
  int SI = 0;
  std::vector<int> q;      // [n_boxes] index of a box's data or -1
  std::vector<int> ids;    // [n] electrode boxes, level order
  std::vector<double> v;   // [n][2D+1][SI]
  std::vector<double> f;   // [n][SI]
  std::vector<double> bv;  // [n][SI]
  std::vector<double> bcc; // [n][SI]
  std::vector<double> dd;  // [n][2D][SI]
  int of(int id) const { return q[id - 1]; }
};

struct Mg {
  afg_mg_desc d;
  std::shared_ptr<Lsf> lsf;  // electrode (null: none)
  int n_coarse = 0;                // unknowns of the coarse grid
  int gx[3] = {1, 1, 1};           // coarse grid size in cells
  std::vector<double> ainv;        // dense inverse, row-major [n][n]
  std::vector<double> amat;        // the matrix itself (kept for the inexact-solve experiment)
  std::vector<double> bc_to_rhs;   // [box-of-lvl1][nb][nc^(D-1)]
  GcSpec gc() const {
    GcSpec g;
    for (int n = 0; n < 6; n++) { g.bc_type[n] = d.bc_type[n]; g.bc_val[n] = d.bc_val[n]; }
    g.rb = AFG_RB_MG_SIDES;
    return g;
  }
};

struct Oracle {
  Tree t;
  std::map<int, GcSpec> methods;   // per cc variable
  std::map<int, Mg> mg;
};

/* Ghost cells (m_af_ghostcell.f90) */
void gc_box(const Tree& t, double* cc, int id, int iv, const GcSpec& g, bool corners);
void gc_lvl(const Tree& t, double* cc, int lvl, int iv, const GcSpec& g, bool corners);

}  // namespace orc

#endif
