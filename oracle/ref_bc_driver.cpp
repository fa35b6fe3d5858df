// C entry points around the reference's own boundary routines (test
// infrastructure only).  ref_bc.py compiles this file after samrai_stub.h and
// the text of enlightning::setAbsorbingBoundaryConditions and
// enlightning::setPhysicalBoundaryConditions, taken unchanged from the
// reference's enlightning.C.  The entry points take the same arguments as the
// oracle's ora_absorb / ora_phys_bc, so the two can be run on the same arrays
// and compared bit for bit.

std::shared_ptr<tbox::Timer> enlightning::t_absorb = std::make_shared<tbox::Timer>();
std::shared_ptr<tbox::Timer> enlightning::t_bc = std::make_shared<tbox::Timer>();

namespace {

std::shared_ptr<pdat::CellData<double>> cell_data(double* p, int g0, int g1) {
  auto d = std::make_shared<pdat::CellData<double>>();
  d->data = p;
  d->gw = hier::IntVector(g0, g1);
  return d;
}

// One patch of box [if0, il0] x [if1, il1] with ghost width (g0, g1) over the
// caller's arrays (depth-major, SAMRAI layout).
hier::Patch make_patch(const enlightning& E, int if0, int il0, int if1, int il1, int g0, int g1, double* w_n,
                       double* pres, double* temp, double* source) {
  hier::Patch P;
  P.box = hier::Box(hier::Index(if0, if1), hier::Index(il0, il1));
  P.geom = std::make_shared<geom::CartesianPatchGeometry>();
  P.data.push_back({E.p_w_n.get(), cell_data(w_n, g0, g1)});
  P.data.push_back({E.p_pressure.get(), cell_data(pres, g0, g1)});
  P.data.push_back({E.p_temperature.get(), cell_data(temp, g0, g1)});
  P.data.push_back({E.p_source.get(), cell_data(source, g0, g1)});
  return P;
}

}  // namespace

extern "C" {

// bc[4] = L, R, B, T boundary types (10 reflect, 20 absorb).
void ref_absorb(int if0, int il0, int if1, int il1, int g0, int g1, const double* patch_xlo, const double* dx,
                const double* grid_xlo, const double* grid_xhi, const int* bc, double absorb_width, double p0,
                double T0, double rho0, double* w_n, double* pres, double* temp) {
  enlightning E;
  E.p_bc_type_L_int = bc[0];
  E.p_bc_type_R_int = bc[1];
  E.p_bc_type_B_int = bc[2];
  E.p_bc_type_T_int = bc[3];
  E.p_bc_absorb_width = absorb_width;
  E.p_p0 = p0;
  E.p_T0 = T0;
  E.p_rho0 = rho0;
  for (int d = 0; d < 2; ++d) {
    E.p_grid_geometry->xlo[d] = grid_xlo[d];
    E.p_grid_geometry->xhi[d] = grid_xhi[d];
  }
  hier::Patch P = make_patch(E, if0, il0, if1, il1, g0, g1, w_n, pres, temp, nullptr);
  for (int d = 0; d < 2; ++d) {
    P.geom->dx[d] = dx[d];
    P.geom->xlo[d] = patch_xlo[d];
  }
  E.setAbsorbingBoundaryConditions(P);
}

// touches[4] = L, R, B, T: the patch side lies on the domain boundary.
// (fw0, fw1) = ghost width to fill.
void ref_phys_bc(int if0, int il0, int if1, int il1, int g0, int g1, const int* touches, const int* bc, int fw0,
                 int fw1, double* w_n, double* pres, double* temp, double* source) {
  enlightning E;
  E.p_bc_type_L_int = bc[0];
  E.p_bc_type_R_int = bc[1];
  E.p_bc_type_B_int = bc[2];
  E.p_bc_type_T_int = bc[3];
  hier::Patch P = make_patch(E, if0, il0, if1, il1, g0, g1, w_n, pres, temp, source);
  for (int loc = 0; loc < 4; ++loc)
    if (touches[loc]) {
      hier::BoundaryBox b;
      b.codim = 1;
      b.loc = loc;
      P.geom->edges.push_back(b);
    }
  for (int loc = 0; loc < 4; ++loc) {
    const int xs = loc & 1, ys = (loc >> 1) & 1;
    if (touches[xs ? 1 : 0] || touches[ys ? 3 : 2]) {
      hier::BoundaryBox b;
      b.codim = 2;
      b.loc = loc;
      P.geom->nodes.push_back(b);
    }
  }
  E.setPhysicalBoundaryConditions(P, 0.0, hier::IntVector(fw0, fw1));
}

}  // extern "C"
