// Mesh construction for the k-eigenvalue path.
//
// CartesianMesh (CartesianMesh.cxx:4-414): cells in x-fastest order, void cells
// (material 0 in the file) dropped, per-cell faces in the order -y, +x, +y, -x, -z, +z
// (2D drops z, 1D drops y), boundary faces carry -(boundary index)-1 with the boundary
// of the face's direction, also where the neighbour is void.  Missing axes use the
// reference's defaults dy = dz = {0.0} (CartesianMesh.hxx), so those coordinates are 0.
//
// UnstructuredExtrudedMesh (UnstructuredExtrudedMesh.cxx:4-364): polygon prisms with
// shoelace area/centroid (math.cxx:4-36), lateral faces in polygon-edge order with the
// (dy, -dx) unit normal (math.cxx:65-79), then -z and +z.  The xy neighbour of an edge is
// found through point -> cell/boundary lists exactly as the reference does, including
// its "last match wins" order and the default boundary for unmatched edges.
//
// split_materials (Mesh.cxx:8-60) and remove_bc_materials (Mesh.cxx:63-204) follow the
// reference; the MPI partitioning of Mesh.cxx:207-394 has no counterpart (one GPU).
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>

#include "pg_host.hpp"

namespace pg {

void Mesh::allocate(int n, int F) {
  num_cells = n;
  fmax = F;
  volumes.assign(n, 0.0);
  centroids.assign((size_t)n * 3, 0.0);
  materials.assign(n, 0);
  num_faces.assign(n, 0);
  areas.assign((size_t)n * F, 0.0);
  fcent.assign((size_t)n * F * 3, 0.0);
  normals.assign((size_t)n * F * 3, 0.0);
  neighbors.assign((size_t)n * F, NO_FACE);
}

namespace {

int read_axis(const std::vector<std::string>& line, Tokens& tok, int& n, std::vector<double>& d) {
  PG_CHECK(line.size() != 2, "wrong number of arguments for keyword '" + line[0] + "'");
  PG_TRY(to_int(line[1], -INT_MAX, INT_MAX, n), "wrong n value");
  if (n > 0) {
    PG_TRY(tok.read_doubles(d, n, 0.0, DBL_MAX), "wrong " + line[0] + " data");
  } else {
    PG_TRY(tok.read_doubles(d, 1, 0.0, DBL_MAX), "wrong " + line[0] + " data");
    n = -n;
    d.assign(n, d[0]);
  }
  return 0;
}

int find_boundary(const std::vector<std::string>& b, const std::string& name) {
  for (size_t i = 0; i < b.size(); i++)
    if (b[i] == name) return (int)i;
  return -1;
}

}  // namespace

int read_cartesian_mesh(const std::string& path, Mesh& mesh) {
  Tokens tok;
  PG_TRY(tok.open(path), "unable to open " + path);
  int nx = 1, ny = 0, nz = 0, num_dims = 0;
  std::vector<double> dx{1.0}, dy{0.0}, dz{0.0};
  std::vector<int> mats;
  std::vector<std::string> boundaries;
  std::map<int, BoundaryCondition> bcs;
  bool has_bcs = false;
  while (true) {
    std::vector<std::string> line = tok.next();
    if (line.empty()) break;
    const std::string& k = line[0];
    if (k == "dx") {
      PG_TRY(read_axis(line, tok, nx, dx), "wrong dx");
      num_dims++;
      boundaries.push_back("-x");
      boundaries.push_back("+x");
    } else if (k == "dy") {
      PG_TRY(read_axis(line, tok, ny, dy), "wrong dy");
      if (ny > 1) num_dims++;
      boundaries.push_back("-y");
      boundaries.push_back("+y");
    } else if (k == "dz") {
      PG_TRY(read_axis(line, tok, nz, dz), "wrong dz");
      if (nz > 1) num_dims++;
      boundaries.push_back("-z");
      boundaries.push_back("+z");
    } else if (k == "bc") {
      PG_CHECK(line.size() < 3, "wrong number of arguments for keyword 'bc'");
      int ibc = find_boundary(boundaries, line[1]);
      PG_CHECK(ibc < 0, "wrong boundary name");
      has_bcs = true;
      PG_TRY(read_bc(line, 2, tok, bcs[ibc + 1]), "wrong boundary condition");
    } else if (k == "materials") {
      int nc = nx * std::max(ny, 1) * std::max(nz, 1), nm;
      PG_TRY(to_int(line.at(1), nc, nc, nm), "wrong number of materials");
      PG_TRY(tok.read_ints(mats, nc, 0, INT_MAX), "wrong material data");
      for (auto& m : mats) m--;
    } else if (k == "nodal-indices") {
      int nc = nx * std::max(ny, 1) * std::max(nz, 1), ni;
      std::vector<int> tmp;
      PG_TRY(to_int(line.at(1), nc, nc, ni), "wrong number of nodal indices");
      PG_TRY(tok.read_ints(tmp, nc, -INT_MAX, INT_MAX), "wrong nodal-index data");
    } else {
      PG_CHECK(true, "unrecognized keyword '" + k + "'");
    }
  }
  const int NY = std::max(ny, 1), NZ = std::max(nz, 1);
  PG_CHECK((int)mats.size() != nx * NY * NZ, "missing material data");
  std::vector<double> x(nx + 1, 0.0), y(ny + 1, 0.0), z(nz + 1, 0.0);
  for (int i = 0; i < nx; i++) x[i + 1] = x[i] + dx[i];
  for (int j = 0; j < ny; j++) y[j + 1] = y[j] + dy[j];
  for (int k = 0; k < nz; k++) z[k + 1] = z[k] + dz[k];

  // compact numbering of physical cells; void pattern must repeat in every layer
  std::vector<int> cid((size_t)nx * NY * NZ, -1);
  int n = 0;
  for (int k = 0; k < NZ; k++)
    for (int j = 0; j < NY; j++)
      for (int i = 0; i < nx; i++) {
        size_t im = ((size_t)k * NY + j) * nx + i;
        if (k > 0) {
          bool v0 = mats[im - (size_t)nx * NY] == -1, v = mats[im] == -1;
          PG_CHECK(v0 != v, "wrong material definition");
        }
        if (mats[im] != -1) cid[im] = n++;
      }
  const int F = (nz > 0) ? 6 : (ny > 0) ? 4 : 2;
  mesh = Mesh();
  mesh.allocate(n, F);
  mesh.num_dims = num_dims;
  // points and cell points (CartesianMesh.cxx:146-228): the whole grid's points, each
  // physical cell's 2, 4 or 8 points in gmsh order
  for (int k = 0; k < nz + 1; k++)
    for (int j = 0; j < ny + 1; j++)
      for (int i = 0; i < nx + 1; i++) {
        mesh.points.push_back(x[i]);
        mesh.points.push_back(y[j]);
        mesh.points.push_back(z[k]);
      }
  for (int k = 0; k < NZ; k++)
    for (int j = 0; j < NY; j++)
      for (int i = 0; i < nx; i++) {
        if (cid[((size_t)k * NY + j) * nx + i] < 0) continue;
        const int sy = nx + 1, sz = (nx + 1) * (ny + 1);
        mesh.cell_pts.push_back(i + j * sy + k * sz);
        mesh.cell_pts.push_back(i + 1 + j * sy + k * sz);
        if (ny > 0) {
          mesh.cell_pts.push_back(i + 1 + (j + 1) * sy + k * sz);
          mesh.cell_pts.push_back(i + (j + 1) * sy + k * sz);
          if (nz > 0) {
            mesh.cell_pts.push_back(i + j * sy + (k + 1) * sz);
            mesh.cell_pts.push_back(i + 1 + j * sy + (k + 1) * sz);
            mesh.cell_pts.push_back(i + 1 + (j + 1) * sy + (k + 1) * sz);
            mesh.cell_pts.push_back(i + (j + 1) * sy + (k + 1) * sz);
          }
        }
        mesh.cell_pts_ptr.push_back((int)mesh.cell_pts.size());
      }
  mesh.boundaries = boundaries;
  mesh.bcs = bcs;
  mesh.has_bcs = has_bcs;
  if (n == nx * NY * NZ && nz > 0) {  // full 3D box: the GPU may sweep it in tiles
    mesh.cart_nx = nx;
    mesh.cart_ny = NY;
    mesh.cart_nz = NZ;
  }
  std::vector<std::string> dirs{"-x", "+x"};
  if (ny > 0) { dirs.push_back("-y"); dirs.push_back("+y"); }
  if (nz > 0) { dirs.push_back("-z"); dirs.push_back("+z"); }
  std::map<std::string, int> bidx;
  for (const auto& d : dirs) {
    int b = find_boundary(boundaries, d);
    PG_CHECK(b < 0, "wrong boundary name");
    bidx[d] = b;
  }
  for (int k = 0; k < NZ; k++)
    for (int j = 0; j < NY; j++)
      for (int i = 0; i < nx; i++) {
        size_t im = ((size_t)k * NY + j) * nx + i;
        int ic = cid[im];
        if (ic < 0) continue;
        mesh.materials[ic] = mats[im];
        mesh.volumes[ic] = (nz > 0) ? dx[i] * dy[j] * dz[k] : (ny > 0) ? dx[i] * dy[j] : dx[i];
        double cx = x[i] + 0.5 * dx[i], cy = y[j] + 0.5 * dy[j], cz = z[k] + 0.5 * dz[k];
        mesh.centroids[(size_t)ic * 3 + 0] = cx;
        mesh.centroids[(size_t)ic * 3 + 1] = cy;
        mesh.centroids[(size_t)ic * 3 + 2] = cz;
        mesh.num_faces[ic] = F;
        auto neighbor = [&](int di, int dj, int dk, const char* name) {
          int i2 = i + di, j2 = j + dj, k2 = k + dk;
          if (i2 < 0 || i2 >= nx || j2 < 0 || j2 >= NY || k2 < 0 || k2 >= NZ) return -bidx[name] - 1;
          int c = cid[((size_t)k2 * NY + j2) * nx + i2];
          return c >= 0 ? c : -bidx[name] - 1;
        };
        auto set = [&](int f, double a, double fx, double fy, double fz, double n0, double n1,
                       double n2, int nb) {
          size_t o = (size_t)ic * F + f;
          mesh.areas[o] = a;
          mesh.fcent[o * 3 + 0] = fx;
          mesh.fcent[o * 3 + 1] = fy;
          mesh.fcent[o * 3 + 2] = fz;
          mesh.normals[o * 3 + 0] = n0;
          mesh.normals[o * 3 + 1] = n1;
          mesh.normals[o * 3 + 2] = n2;
          mesh.neighbors[o] = nb;
        };
        const double ax = (nz > 0) ? dy[j] * dz[k] : (ny > 0) ? dy[j] : 1.0;
        const double ay = (nz > 0) ? dx[i] * dz[k] : dx[i];
        int f = 0;
        if (ny > 0) set(f++, ay, cx, y[j], cz, 0.0, -1.0, 0.0, neighbor(0, -1, 0, "-y"));
        set(f++, ax, x[i] + dx[i], cy, cz, 1.0, 0.0, 0.0, neighbor(1, 0, 0, "+x"));
        if (ny > 0) set(f++, ay, cx, y[j] + dy[j], cz, 0.0, 1.0, 0.0, neighbor(0, 1, 0, "+y"));
        set(f++, ax, x[i], cy, cz, -1.0, 0.0, 0.0, neighbor(-1, 0, 0, "-x"));
        if (nz > 0) {
          set(f++, dx[i] * dy[j], cx, cy, z[k], 0.0, 0.0, -1.0, neighbor(0, 0, -1, "-z"));
          set(f++, dx[i] * dy[j], cx, cy, z[k] + dz[k], 0.0, 0.0, 1.0, neighbor(0, 0, 1, "+z"));
        }
      }
  return 0;
}

namespace {

double poly_area(const std::vector<double>& pts, const std::vector<int>& ids) {
  double a = 0.0;
  const size_t n = ids.size();
  for (size_t q = 0; q < n; q++) {
    const double* p1 = &pts[(size_t)ids[q] * 2];
    const double* p2 = &pts[(size_t)ids[(q + 1) % n] * 2];
    a += p1[0] * p2[1] - p2[0] * p1[1];
  }
  return a * 0.5;
}

void poly_centroid(const std::vector<double>& pts, const std::vector<int>& ids, double a, double* c) {
  double c0 = 0.0, c1 = 0.0;
  const size_t n = ids.size();
  for (size_t q = 0; q < n; q++) {
    const double* p1 = &pts[(size_t)ids[q] * 2];
    const double* p2 = &pts[(size_t)ids[(q + 1) % n] * 2];
    double da = p1[0] * p2[1] - p2[0] * p1[1];
    c0 += (p1[0] + p2[0]) * da;
    c1 += (p1[1] + p2[1]) * da;
  }
  c[0] = c0 * (1.0 / (6.0 * a));
  c[1] = c1 * (1.0 / (6.0 * a));
}

}  // namespace

int read_unstructured_mesh(const std::string& path, Mesh& mesh) {
  Tokens tok;
  PG_TRY(tok.open(path), "unable to open " + path);
  std::vector<double> pts;
  std::vector<std::vector<int>> cells;
  int nz = 0, num_dims = 0, default_b = -1;
  std::vector<double> dz;
  std::vector<std::string> boundaries, xy_bnames;
  std::vector<std::vector<int>> xy_bpoints;
  std::map<int, BoundaryCondition> bcs;
  bool has_bcs = false;
  std::vector<int> mats;
  while (true) {
    std::vector<std::string> line = tok.next();
    if (line.empty()) break;
    const std::string& k = line[0];
    if (k == "points") {
      int np;
      PG_TRY(to_int(line.at(1), 1, INT_MAX, np), "wrong number of points");
      pts.clear();
      for (int p = 0; p < np; p++) {
        std::vector<std::string> row = tok.next();
        PG_CHECK(row.size() != 2, "wrong point data");
        double a, b;
        PG_TRY(to_double(row[0], -DBL_MAX, DBL_MAX, a), "wrong point data");
        PG_TRY(to_double(row[1], -DBL_MAX, DBL_MAX, b), "wrong point data");
        pts.push_back(a);
        pts.push_back(b);
      }
    } else if (k == "cells") {
      int nc, ntot;
      PG_CHECK(line.size() != 3, "wrong number of arguments for keyword 'cells'");
      PG_TRY(to_int(line[1], 1, INT_MAX, nc), "wrong number of cells");
      PG_TRY(to_int(line[2], 1, INT_MAX, ntot), "wrong number of cell points");
      cells.clear();
      size_t tot = 0;
      for (int c = 0; c < nc; c++) {
        std::vector<std::string> row = tok.next();
        PG_CHECK(row.empty(), "missing cell data");
        tot += row.size();
        PG_CHECK(tot > (size_t)ntot, "out-of-bounds cell data");
        std::vector<int> ids;
        for (const auto& w : row) {
          int p;
          PG_TRY(to_int(w, 0, INT_MAX, p), "wrong cell data");
          ids.push_back(p);
        }
        cells.push_back(ids);
      }
      num_dims += 2;
    } else if (k == "dz") {
      PG_TRY(read_axis(line, tok, nz, dz), "wrong dz");
      if (nz > 1) num_dims++;
      boundaries.push_back("-z");
      boundaries.push_back("+z");
    } else if (k == "boundary") {
      PG_CHECK(line.size() != 3, "wrong number of arguments for keyword 'boundary'");
      boundaries.push_back(line[1]);
      xy_bnames.push_back(line[1]);
      int nb;
      PG_TRY(to_int(line[2], 0, INT_MAX, nb), "wrong number of boundary points");
      std::vector<int> bp;
      if (nb > 0) PG_TRY(tok.read_ints(bp, nb, 0, INT_MAX), "wrong boundary data");
      else default_b = (int)xy_bpoints.size();
      xy_bpoints.push_back(bp);
    } else if (k == "bc") {
      PG_CHECK(line.size() < 3, "wrong number of arguments for keyword 'bc'");
      int ibc = find_boundary(boundaries, line[1]);
      PG_CHECK(ibc < 0, "wrong boundary name");
      has_bcs = true;
      PG_TRY(read_bc(line, 2, tok, bcs[ibc + 1]), "wrong boundary condition");
    } else if (k == "materials") {
      int nc = (int)cells.size() * std::max(nz, 1), nm;
      PG_TRY(to_int(line.at(1), nc, nc, nm), "wrong number of materials");
      PG_TRY(tok.read_ints(mats, nc, 0, INT_MAX), "wrong material data");
      for (auto& m : mats) m--;
    } else if (k == "nodal-indices") {
      int nc = (int)cells.size() * std::max(nz, 1), ni;
      std::vector<int> tmp;
      PG_TRY(to_int(line.at(1), nc, nc, ni), "wrong number of nodal indices");
      PG_TRY(tok.read_ints(tmp, nc, -INT_MAX, INT_MAX), "wrong nodal-index data");
    } else {
      PG_CHECK(true, "unrecognized keyword '" + k + "'");
    }
  }
  const int nxy = (int)cells.size();
  const int npts = (int)pts.size() / 2;
  const int NZ = std::max(nz, 1);
  PG_CHECK((int)mats.size() != nxy * NZ, "missing material data");
  if (nz == 0) dz.assign(1, 0.0);
  std::vector<double> z(nz + 1, 0.0);
  for (int k = 0; k < nz; k++) z[k + 1] = z[k] + dz[k];

  std::vector<double> xy_area(nxy), xy_cent((size_t)nxy * 2);
  int nmax = 0;
  for (int i = 0; i < nxy; i++) {
    for (int p : cells[i]) PG_CHECK(p >= npts, "wrong cell point index");
    xy_area[i] = poly_area(pts, cells[i]);
    poly_centroid(pts, cells[i], xy_area[i], &xy_cent[(size_t)i * 2]);
    nmax = std::max(nmax, (int)cells[i].size());
  }
  // point -> cells then boundaries (UnstructuredExtrudedMesh.cxx:227-251)
  std::vector<std::vector<int>> pcells(npts);
  for (int i = 0; i < nxy; i++)
    for (int p : cells[i]) pcells[p].push_back(i);
  for (size_t b = 0; b < xy_bnames.size(); b++) {
    int bi = find_boundary(boundaries, xy_bnames[b]);
    PG_CHECK(bi < 0, "wrong boundary name");
    for (int p : xy_bpoints[b]) {
      PG_CHECK(p >= npts, "wrong boundary point index");
      pcells[p].push_back(-bi - 1);
    }
  }
  std::vector<std::vector<int>> xy_nbr(nxy);
  for (int i = 0; i < nxy; i++) {
    const int nn = (int)cells[i].size();
    xy_nbr[i].assign(nn, 0);
    for (int f = 0; f < nn; f++) {
      int ip1 = cells[i][f], ip2 = cells[i][(f + 1) % nn];
      bool found = false;
      int val = 0;
      for (int i1 : pcells[ip1])
        for (int i2 : pcells[ip2])
          if (i1 == i2 && i1 != i) {
            PG_CHECK(found && val > 0, "wrong mesh connectivity");
            val = i1;
            found = true;
          }
      if (!found && default_b >= 0) {
        // The reference stores the position of the default boundary among the xy
        // boundaries (UnstructuredExtrudedMesh.cxx:86, 271-274), not its index in the
        // full boundary list; kept as is.
        val = -default_b - 1;
        found = true;
      }
      PG_CHECK(!found, "wrong mesh connectivity");
      xy_nbr[i][f] = val;
    }
  }
  const int F = (nz > 0) ? nmax + 2 : nmax;
  mesh = Mesh();
  mesh.allocate(nxy * NZ, F);
  mesh.num_dims = num_dims;
  // points and cell points (UnstructuredExtrudedMesh.cxx:153-201): the xy points on every
  // z level; a cell's polygon on its lower level, then on its upper level
  for (int k = 0; k < nz + 1; k++)
    for (int p = 0; p < npts; p++) {
      mesh.points.push_back(pts[(size_t)p * 2]);
      mesh.points.push_back(pts[(size_t)p * 2 + 1]);
      mesh.points.push_back(z[k]);
    }
  for (int k = 0; k < NZ; k++)
    for (int i = 0; i < nxy; i++) {
      for (int p : cells[i]) mesh.cell_pts.push_back(p + k * npts);
      if (nz > 0)
        for (int p : cells[i]) mesh.cell_pts.push_back(p + (k + 1) * npts);
      mesh.cell_pts_ptr.push_back((int)mesh.cell_pts.size());
    }
  mesh.boundaries = boundaries;
  mesh.bcs = bcs;
  mesh.has_bcs = has_bcs;
  int bzm = -1, bzp = -1;
  if (nz > 0) {
    bzm = find_boundary(boundaries, "-z");
    bzp = find_boundary(boundaries, "+z");
  }
  int ic = 0;
  for (int k = 0; k < NZ; k++) {
    const double zmid = z[k] + 0.5 * dz[k];
    for (int i = 0; i < nxy; i++, ic++) {
      const int nn = (int)cells[i].size();
      const double a = xy_area[i];
      mesh.materials[ic] = mats[ic];
      mesh.volumes[ic] = (nz > 0) ? a * dz[k] : a;
      mesh.centroids[(size_t)ic * 3 + 0] = xy_cent[(size_t)i * 2];
      mesh.centroids[(size_t)ic * 3 + 1] = xy_cent[(size_t)i * 2 + 1];
      mesh.centroids[(size_t)ic * 3 + 2] = zmid;
      mesh.num_faces[ic] = (nz > 0) ? nn + 2 : nn;
      for (int f = 0; f < nn; f++) {
        const double* p1 = &pts[(size_t)cells[i][f] * 2];
        const double* p2 = &pts[(size_t)cells[i][(f + 1) % nn] * 2];
        size_t o = (size_t)ic * F + f;
        double d = std::sqrt(std::pow(p2[0] - p1[0], 2) + std::pow(p2[1] - p1[1], 2));
        mesh.areas[o] = (nz > 0) ? d * dz[k] : d;
        mesh.fcent[o * 3 + 0] = 0.5 * (p1[0] + p2[0]);
        mesh.fcent[o * 3 + 1] = 0.5 * (p1[1] + p2[1]);
        mesh.fcent[o * 3 + 2] = zmid;
        double n0 = p2[1] - p1[1], n1 = p1[0] - p2[0];
        double nr = std::sqrt(n0 * n0 + n1 * n1);
        mesh.normals[o * 3 + 0] = n0 / nr;
        mesh.normals[o * 3 + 1] = n1 / nr;
        mesh.normals[o * 3 + 2] = 0.0;
        int j = xy_nbr[i][f];
        mesh.neighbors[o] = j >= 0 ? j + k * nxy : j;
      }
      if (nz > 0) {
        for (int s = 0; s < 2; s++) {
          size_t o = (size_t)ic * F + nn + s;
          mesh.areas[o] = a;
          mesh.fcent[o * 3 + 0] = xy_cent[(size_t)i * 2];
          mesh.fcent[o * 3 + 1] = xy_cent[(size_t)i * 2 + 1];
          mesh.fcent[o * 3 + 2] = s == 0 ? z[k] : z[k] + dz[k];
          mesh.normals[o * 3 + 2] = s == 0 ? -1.0 : 1.0;
          if (s == 0) mesh.neighbors[o] = (k == 0) ? -bzm - 1 : ic - nxy;
          else mesh.neighbors[o] = (k == nz - 1) ? -bzp - 1 : ic + nxy;
        }
      }
    }
  }
  return 0;
}

int split_materials(Mesh& mesh, std::vector<Material>& materials) {
  for (int i = 0; i < mesh.num_cells; i++) {
    const int im = mesh.materials[i];
    if (!materials[im].split) continue;
    const int im2 = (int)materials.size();
    std::vector<int> stack{i};
    mesh.materials[i] = im2;
    while (!stack.empty()) {
      int c = stack.back();
      stack.pop_back();
      for (int f = 0; f < mesh.num_faces[c]; f++) {
        int c2 = mesh.nbr(c, f);
        if (c2 >= 0 && mesh.materials[c2] == im) {
          mesh.materials[c2] = im2;
          stack.push_back(c2);
        }
      }
    }
    Material sub = materials[im];
    sub.name = materials[im].name + "-" + std::to_string(materials[im].num_sub);
    sub.split = false;
    sub.num_sub = 0;
    materials[im].num_sub++;
    if (sub.bc) mesh.boundaries.push_back(sub.name);
    materials.push_back(sub);
  }
  return 0;
}

int remove_bc_materials(const Mesh& in, const std::vector<Material>& materials, Mesh& out) {
  const int n0 = in.num_cells;
  std::vector<int> newid(n0, -1);
  int n = 0, F = 0;
  for (int i = 0; i < n0; i++)
    if (!materials[in.materials[i]].bc) {
      newid[i] = n++;
      F = std::max(F, in.num_faces[i]);
    }
  std::vector<int> matb(materials.size(), -1);
  for (size_t m = 0; m < materials.size(); m++)
    if (materials[m].bc) {
      matb[m] = find_boundary(in.boundaries, materials[m].name);
      PG_CHECK(matb[m] < 0, "wrong boundary name");
    }
  out = Mesh();
  out.allocate(n, F);
  out.num_dims = in.num_dims;
  out.boundaries = in.boundaries;
  out.bcs = in.bcs;
  out.has_bcs = in.has_bcs;
  // points used by the remaining cells, renumbered in order (Mesh.cxx:91-114)
  if ((int)in.cell_pts_ptr.size() == n0 + 1) {
    const int np = (int)in.points.size() / 3;
    std::vector<int> used(np, 0), ip(np, -1);
    for (int i = 0; i < n0; i++)
      if (newid[i] >= 0)
        for (int k = in.cell_pts_ptr[i]; k < in.cell_pts_ptr[i + 1]; k++) used[in.cell_pts[k]] = 1;
    for (int p = 0, q = 0; p < np; p++)
      if (used[p]) {
        ip[p] = q++;
        for (int d = 0; d < 3; d++) out.points.push_back(in.points[(size_t)p * 3 + d]);
      }
    for (int i = 0; i < n0; i++)
      if (newid[i] >= 0) {
        for (int k = in.cell_pts_ptr[i]; k < in.cell_pts_ptr[i + 1]; k++) out.cell_pts.push_back(ip[in.cell_pts[k]]);
        out.cell_pts_ptr.push_back((int)out.cell_pts.size());
      }
  }
  for (int i = 0; i < n0; i++) {
    int ic = newid[i];
    if (ic < 0) continue;
    out.volumes[ic] = in.volumes[i];
    for (int d = 0; d < 3; d++) out.centroids[(size_t)ic * 3 + d] = in.centroids[(size_t)i * 3 + d];
    out.materials[ic] = in.materials[i];
    out.num_faces[ic] = in.num_faces[i];
    for (int f = 0; f < in.num_faces[i]; f++) {
      size_t o = (size_t)ic * F + f, oi = (size_t)i * in.fmax + f;
      out.areas[o] = in.areas[oi];
      for (int d = 0; d < 3; d++) {
        out.fcent[o * 3 + d] = in.fcent[oi * 3 + d];
        out.normals[o * 3 + d] = in.normals[oi * 3 + d];
      }
      int i2 = in.neighbors[oi];
      if (i2 >= 0) out.neighbors[o] = materials[in.materials[i2]].bc ? -matb[in.materials[i2]] - 1 : newid[i2];
      else out.neighbors[o] = i2;
    }
  }
  return 0;
}

}  // namespace pg
