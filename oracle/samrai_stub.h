// Minimal stand-ins for the SAMRAI v3 types that the reference's two
// boundary routines use, so that those routines compile unchanged from the
// reference's own source text (test infrastructure only; see ref_bc.py).
//
// SAMRAI itself is not available here.  What this file restates of it:
//   * hier::Box / Index / IntVector: cell-centred index boxes, indexed as
//     box.lower()(d) and box.upper()(d);
//   * pdat::CellData<double>: a depth-major array over the patch box grown by
//     its ghost width (getPointer, getGhostCellWidth);
//   * geom::CartesianPatchGeometry: dx, the patch's lower corner, and the
//     boundary boxes of a patch in a single-box, non-periodic domain:
//       - an edge box (codimension 1) on every side of the patch that lies on
//         the domain boundary, location index 0 = x lower, 1 = x upper,
//         2 = y lower, 3 = y upper, in that order;
//       - a node box (codimension 2) at every corner of the patch whose
//         diagonal ghost region lies outside the domain, that is, next to at
//         least one such side; location index 0 = (x lo, y lo),
//         1 = (x hi, y lo), 2 = (x lo, y hi), 3 = (x hi, y hi);
//     and getBoundaryFillBox: the part of the patch's ghost region of the
//     given width that the boundary box covers (edge boxes span the patch
//     interior tangentially, node boxes the ghost corner);
//   * the patch-strategy members the routines read (boundary types, ambient
//     state, absorbing width, the grid's extent) as plain fields.
#pragma once

#include <cmath>
#include <cstdio>
#include <memory>
#include <string>
#include <vector>

namespace boost {
using std::shared_ptr;
}
#define BOOST_CAST std::static_pointer_cast

// enlightning.C's interface constants (boundary types, state depth, square)
#define NEQU (5)
#define REFLECT (10)
#define ABSORB (20)
#define SQUARE(x) ((x) * (x))

namespace SAMRAI {
namespace tbox {
struct Timer {
  void start() {}
  void stop() {}
};
}  // namespace tbox

namespace hier {
struct IntVector {
  int v[2];
  IntVector(int a = 0, int b = 0) : v{a, b} {}
  int operator()(int d) const { return v[d]; }
};
struct Index {
  int v[2];
  Index(int a = 0, int b = 0) : v{a, b} {}
  int operator()(int d) const { return v[d]; }
};
struct Box {
  Index lo, hi;
  Box() : lo(0, 0), hi(-1, -1) {}
  Box(const Index& l, const Index& h) : lo(l), hi(h) {}
  const Index& lower() const { return lo; }
  const Index& upper() const { return hi; }
};
struct BoundaryBox {
  Box box;
  int codim = 1;
  int loc = 0;
  int getLocationIndex() const { return loc; }
};
struct PatchData {
  virtual ~PatchData() {}
};
struct PatchGeometry {
  virtual ~PatchGeometry() {}
};
struct VariableContext {};
}  // namespace hier

namespace pdat {
template <typename T>
struct CellVariable {};
template <typename T>
struct CellData : hier::PatchData {
  T* data = nullptr;
  hier::IntVector gw;
  T* getPointer() { return data; }
  hier::IntVector getGhostCellWidth() const { return gw; }
};
}  // namespace pdat

namespace geom {
struct CartesianGridGeometry {
  double xlo[2], xhi[2];
  const double* getXLower() const { return xlo; }
  const double* getXUpper() const { return xhi; }
};
struct CartesianPatchGeometry : hier::PatchGeometry {
  double dx[2], xlo[2];
  std::vector<hier::BoundaryBox> edges, nodes;
  const double* getDx() const { return dx; }
  const double* getXLower() const { return xlo; }
  std::vector<hier::BoundaryBox> getEdgeBoundaries() const { return edges; }
  std::vector<hier::BoundaryBox> getNodeBoundaries() const { return nodes; }
  // The ghost cells of width gw that boundary box b covers.
  hier::Box getBoundaryFillBox(const hier::BoundaryBox& b, const hier::Box& patch,
                               const hier::IntVector& gw) const {
    int lo[2], hi[2];
    for (int d = 0; d < 2; ++d) {
      lo[d] = patch.lower()(d);
      hi[d] = patch.upper()(d);
    }
    // side of the patch in each direction: -1 lower, +1 upper, 0 spanning
    int side[2] = {0, 0};
    if (b.codim == 1) {
      side[b.loc / 2] = (b.loc % 2) ? 1 : -1;
    } else {
      side[0] = (b.loc & 1) ? 1 : -1;
      side[1] = (b.loc & 2) ? 1 : -1;
    }
    int flo[2], fhi[2];
    for (int d = 0; d < 2; ++d) {
      if (side[d] < 0) {
        flo[d] = lo[d] - gw(d);
        fhi[d] = lo[d] - 1;
      } else if (side[d] > 0) {
        flo[d] = hi[d] + 1;
        fhi[d] = hi[d] + gw(d);
      } else {
        flo[d] = lo[d];
        fhi[d] = hi[d];
      }
    }
    return hier::Box(hier::Index(flo[0], flo[1]), hier::Index(fhi[0], fhi[1]));
  }
};
}  // namespace geom

namespace hier {
// A patch: its box, its geometry and the four cell arrays the routines read,
// looked up by the variable they belong to.
struct Patch {
  Box box;
  std::shared_ptr<geom::CartesianPatchGeometry> geom;
  std::vector<std::pair<const void*, std::shared_ptr<pdat::CellData<double>>>> data;
  const Box& getBox() const { return box; }
  std::shared_ptr<PatchGeometry> getPatchGeometry() const { return geom; }
  std::shared_ptr<PatchData> getPatchData(const std::shared_ptr<pdat::CellVariable<double>>& var,
                                          const std::shared_ptr<VariableContext>&) const {
    for (auto& e : data)
      if (e.first == var.get()) return e.second;
    std::fprintf(stderr, "samrai_stub: unknown variable\n");
    return nullptr;
  }
};
}  // namespace hier
}  // namespace SAMRAI

using namespace SAMRAI;
using std::string;

// The members of the reference's patch strategy that the two routines use.
class enlightning {
 public:
  void setPhysicalBoundaryConditions(hier::Patch& patch, const double fill_time,
                                     const hier::IntVector& ghost_width_to_fill);
  void setAbsorbingBoundaryConditions(hier::Patch& patch) const;

  std::shared_ptr<hier::VariableContext> getInteriorWithGhostsContext() const { return ctx; }

  std::shared_ptr<hier::VariableContext> ctx = std::make_shared<hier::VariableContext>();
  std::shared_ptr<geom::CartesianGridGeometry> p_grid_geometry = std::make_shared<geom::CartesianGridGeometry>();
  std::shared_ptr<pdat::CellVariable<double>> p_w_n = std::make_shared<pdat::CellVariable<double>>();
  std::shared_ptr<pdat::CellVariable<double>> p_pressure = std::make_shared<pdat::CellVariable<double>>();
  std::shared_ptr<pdat::CellVariable<double>> p_temperature = std::make_shared<pdat::CellVariable<double>>();
  std::shared_ptr<pdat::CellVariable<double>> p_source = std::make_shared<pdat::CellVariable<double>>();
  int p_bc_type_L_int = REFLECT, p_bc_type_R_int = REFLECT, p_bc_type_B_int = REFLECT, p_bc_type_T_int = REFLECT;
  double p_bc_absorb_width = 0.0;
  double p_p0 = 0.0, p_T0 = 0.0, p_rho0 = 0.0;
  static std::shared_ptr<tbox::Timer> t_absorb;
  static std::shared_ptr<tbox::Timer> t_bc;
};
