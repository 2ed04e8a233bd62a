// Side outputs of a solve: the .vtk files of vtk.cxx (mesh with materials, then the
// solution fields appended) and the PETSc binary dump of petsc::write (petsc.cxx:491-511).
// Both are off unless switched on, as in the reference (-vtk, -vtk_interval, -petsc_dump,
// or the input's `vtk` / `petsc dump` keywords).
#include <cstdint>
#include <cstring>
#include <fstream>
#include <iomanip>

#include "pg_host.hpp"

namespace pg {

namespace {

// vtk::write's file name: prefix_<n / interval>.vtk (vtk.cxx:37, 134).
std::string vtk_name(const std::string& prefix, int n, int dn) { return prefix + "_" + std::to_string(n / dn) + ".vtk"; }

// VTK cell type of a cell with np points (vtk.cxx:82-97): line, triangle, quad, wedge,
// hexahedron, hexagonal prism.
int vtk_cell_type(int np) {
  switch (np) {
    case 2: return 3;
    case 3: return 5;
    case 4: return 9;
    case 6: return 13;
    case 8: return 12;
    case 12: return 16;
    default: return -1;
  }
}

void put_be32(std::ofstream& f, uint32_t v) {
  unsigned char b[4] = {(unsigned char)(v >> 24), (unsigned char)(v >> 16), (unsigned char)(v >> 8), (unsigned char)v};
  f.write(reinterpret_cast<const char*>(b), 4);
}

}  // namespace

// vtk::write for the mesh (vtk.cxx:28-121): header, points, cells, cell types, materials.
int write_vtk_mesh(const std::string& prefix, int n, const RunOptions& opt, const Mesh& mesh) {
  if (!opt.vtk || n % opt.vtk_interval != 0) return 0;
  const std::string name = vtk_name(prefix, n, opt.vtk_interval);
  std::ofstream f(name, std::ios_base::out);
  PG_CHECK(!f.is_open(), "unable to open " + name);
  const int np = (int)mesh.points.size() / 3, nc = mesh.num_cells;
  PG_CHECK((int)mesh.cell_pts_ptr.size() != nc + 1, "the mesh has no point data for the .vtk output");
  f << std::scientific << std::setprecision(6);
  f << "# vtk DataFile Version 3.0\nFVM mesh\nASCII\nDATASET UNSTRUCTURED_GRID\n\n";
  f << "POINTS " << np << " double\n";
  for (int p = 0; p < np; p++)
    f << mesh.points[(size_t)p * 3] << " " << mesh.points[(size_t)p * 3 + 1] << " " << mesh.points[(size_t)p * 3 + 2]
      << "\n";
  f << "\n";
  f << "CELLS " << nc << " " << nc + mesh.cell_pts_ptr[nc] << "\n";
  for (int i = 0; i < nc; i++) {
    f << mesh.cell_pts_ptr[i + 1] - mesh.cell_pts_ptr[i];
    for (int k = mesh.cell_pts_ptr[i]; k < mesh.cell_pts_ptr[i + 1]; k++) f << " " << mesh.cell_pts[k];
    f << "\n";
  }
  f << "\n";
  f << "CELL_TYPES " << nc << "\n";
  for (int i = 0; i < nc; i++) {
    const int t = vtk_cell_type(mesh.cell_pts_ptr[i + 1] - mesh.cell_pts_ptr[i]);
    PG_CHECK(t < 0, "wrong cell type");
    f << t << "\n";
  }
  f << "\n";
  f << "CELL_DATA " << nc << "\n\n";
  f << "SCALARS materials double 1\nLOOKUP_TABLE default\n";
  for (int i = 0; i < nc; i++) f << mesh.materials[i] + 1 << "\n";
  f << "\n";
  PG_CHECK(!f.good(), "unable to write " + name);
  return 0;
}

// vtk::write for a solution vector (vtk.cxx:123-170): one section per group and direction,
// v[(i*G + g)*M + m].
int write_vtk_field(const std::string& prefix, int n, const RunOptions& opt, const std::string& name,
                    const std::vector<double>& v, int num_cells, int num_groups, int num_directions) {
  if (!opt.vtk || n % opt.vtk_interval != 0) return 0;
  const std::string file = vtk_name(prefix, n, opt.vtk_interval);
  std::ofstream f(file, std::ios_base::app);
  PG_CHECK(!f.is_open(), "unable to open " + file);
  PG_CHECK(v.size() < (size_t)num_cells * num_groups * num_directions, "field smaller than the mesh");
  f << std::scientific << std::setprecision(6);
  const size_t div = (size_t)num_groups * num_directions;
  for (int g = 0; g < num_groups; g++)
    for (int m = 0; m < num_directions; m++) {
      f << "SCALARS " << name;
      if (num_groups > 1) f << "_" << (g + 1);
      if (num_directions > 1) f << "_" << (m + 1);
      f << " double 1\nLOOKUP_TABLE default\n";
      for (size_t iv = (size_t)g * num_directions + m, i = 0; i < (size_t)num_cells; i++, iv += div) f << v[iv] << "\n";
      f << "\n";
    }
  PG_CHECK(!f.good(), "unable to write " + file);
  return 0;
}

// petsc::write (petsc.cxx:491-511): VecView to a binary viewer, i.e. the vector class id
// 1211214 and the length as big-endian 32-bit integers, then the values as big-endian
// doubles, in prefix_<n>.ptc; the viewer also creates an (empty) prefix_<n>.ptc.info.
int write_petsc_vec(const std::string& prefix, int n, const RunOptions& opt, const std::vector<double>& v) {
  if (!opt.dump) return 0;
  const std::string name = prefix + "_" + std::to_string(n) + ".ptc";
  std::ofstream f(name, std::ios_base::out | std::ios_base::binary);
  PG_CHECK(!f.is_open(), "unable to open " + name);
  put_be32(f, 1211214u);
  put_be32(f, (uint32_t)v.size());
  for (double x : v) {
    uint64_t u;
    std::memcpy(&u, &x, 8);
    put_be32(f, (uint32_t)(u >> 32));
    put_be32(f, (uint32_t)u);
  }
  PG_CHECK(!f.good(), "unable to write " + name);
  std::ofstream info(name + ".info", std::ios_base::out);
  PG_CHECK(!info.is_open(), "unable to open " + name + ".info");
  return 0;
}

}  // namespace pg
