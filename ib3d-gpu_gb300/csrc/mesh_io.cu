// Surface-mesh files and force-driven body motion.
//
// readSurfaceMeshGmsh (subReadInput.f90:137-176) and readSurfaceMeshGambit
// (:180-213) read the body's triangulation with list-directed READs, one record per
// READ statement: Gmsh 2 skips 4 lines, reads the node count, the nodes
// "id x y z", skips 2 lines, reads the element count, skips surGeoPoints element
// lines and takes the last three of the eight integers of each remaining line;
// Gambit skips 6 lines, reads "NUMNP NELEM ...", skips 2, reads the nodes
// "id x y z", skips 2, reads the elements "id type n n1 n2 n3". The readers below
// follow the same record structure (blank- or comma-separated fields).
//
// shiftSurfaceNodesMovingbody (subSearch.f90:41-76) integrates the body velocity
// from the surface force: u_final = F/(vol*1)*deltat + u_init with vol the volume
// of a unit-diameter sphere, pi/6, and density 1, then shifts the nodes by
// u_final*deltat. The reference never computes Total_Force_X/Y/Z, so the caller
// supplies the force.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "ib3d_internal.cuh"

namespace {

bool next_line(FILE* fp, std::string& out) {
  out.clear();
  int ch;
  bool any = false;
  while ((ch = std::fgetc(fp)) != EOF) {
    any = true;
    if (ch == '\n') break;
    out.push_back((char)ch);
  }
  return any;
}

// the first n numbers of a list-directed record
bool numbers(const std::string& line, int n, double* out) {
  const char* p = line.c_str();
  for (int q = 0; q < n; ++q) {
    while (*p == ' ' || *p == '\t' || *p == ',' || *p == '\r') ++p;
    char* end = nullptr;
    out[q] = std::strtod(p, &end);
    if (end == p) return false;
    p = end;
  }
  return true;
}

struct Mesh {
  std::vector<double> x, y, z;
  std::vector<int64_t> e1, e2, e3;
};

int read_mesh(const char* path, int format, int64_t sur_geo_points, Mesh& m, std::string& err) {
  FILE* fp = std::fopen(path, "r");
  if (!fp) { err = "cannot open the mesh file"; return IB3D_ERR_IO; }
  std::string ln;
  double v[8];
  auto skip = [&](int n) { for (int q = 0; q < n; ++q) if (!next_line(fp, ln)) return false; return true; };
  auto fail = [&](const char* msg) { std::fclose(fp); err = msg; return IB3D_ERR_IO; };
  int64_t nn = 0, ne = 0;
  if (format == IB3D_MESH_GMSH) {
    if (!skip(4) || !next_line(fp, ln) || !numbers(ln, 1, v)) return fail("Gmsh: no node count");
    nn = (int64_t)v[0];
  } else if (format == IB3D_MESH_GAMBIT) {
    if (!skip(6) || !next_line(fp, ln) || !numbers(ln, 2, v)) return fail("Gambit: no NUMNP/NELEM record");
    nn = (int64_t)v[0];
    ne = (int64_t)v[1];
    if (!skip(2)) return fail("Gambit: truncated before the nodes");
  } else {
    std::fclose(fp);
    err = "unknown mesh format";
    return IB3D_ERR_ARG;
  }
  if (nn < 3 || nn > (1ll << 30)) return fail("bad node count");
  m.x.resize(nn); m.y.resize(nn); m.z.resize(nn);
  for (int64_t n = 0; n < nn; ++n) {
    if (!next_line(fp, ln) || !numbers(ln, 4, v)) return fail("truncated or malformed node record");
    m.x[n] = v[1]; m.y[n] = v[2]; m.z[n] = v[3];
  }
  if (!skip(2)) return fail("truncated before the elements");
  int take = 6;   // Gambit: id type n n1 n2 n3
  if (format == IB3D_MESH_GMSH) {
    if (!next_line(fp, ln) || !numbers(ln, 1, v)) return fail("Gmsh: no element count");
    ne = (int64_t)v[0];
    if (sur_geo_points < 0 || sur_geo_points > ne || !skip((int)sur_geo_points)) return fail("Gmsh: surGeoPoints");
    ne -= sur_geo_points;
    take = 8;     // id type ntags tag1 tag2 n1 n2 n3
  }
  if (ne < 1 || ne > (1ll << 30)) return fail("bad element count");
  m.e1.resize(ne); m.e2.resize(ne); m.e3.resize(ne);
  for (int64_t n = 0; n < ne; ++n) {
    if (!next_line(fp, ln) || !numbers(ln, take, v)) return fail("truncated or malformed element record");
    m.e1[n] = (int64_t)v[take - 3]; m.e2[n] = (int64_t)v[take - 2]; m.e3[n] = (int64_t)v[take - 1];
  }
  std::fclose(fp);
  return IB3D_OK;
}

}  // namespace

extern "C" {

int ib3d_read_surface_mesh(const char* path, int32_t format, int64_t sur_geo_points, int64_t* nnodes, double* xn,
                           double* yn, double* zn, int64_t* nelems, int64_t* e1, int64_t* e2, int64_t* e3) {
  if (!path || !nnodes || !nelems) return IB3D_ERR_ARG;
  Mesh m;
  std::string err;
  const int rc = read_mesh(path, format, sur_geo_points, m, err);
  if (rc) return rc;
  const bool fill = xn && yn && zn && e1 && e2 && e3;
  if (fill && (*nnodes < (int64_t)m.x.size() || *nelems < (int64_t)m.e1.size())) return IB3D_ERR_ARG;
  *nnodes = (int64_t)m.x.size();
  *nelems = (int64_t)m.e1.size();
  if (fill) {
    std::memcpy(xn, m.x.data(), m.x.size() * sizeof(double));
    std::memcpy(yn, m.y.data(), m.y.size() * sizeof(double));
    std::memcpy(zn, m.z.data(), m.z.size() * sizeof(double));
    std::memcpy(e1, m.e1.data(), m.e1.size() * sizeof(int64_t));
    std::memcpy(e2, m.e2.data(), m.e2.size() * sizeof(int64_t));
    std::memcpy(e3, m.e3.data(), m.e3.size() * sizeof(int64_t));
  }
  return IB3D_OK;
}

int ib3d_set_mesh_file(ib3d_ctx* c, const char* path, int32_t format, int64_t sur_geo_points, double xshift,
                       double yshift, double zshift, int64_t inor) {
  if (!c || !path) return IB3D_ERR_ARG;
  Mesh m;
  std::string err;
  const int rc = read_mesh(path, format, sur_geo_points, m, err);
  if (rc) {
    c->err = "ib3d_set_mesh_file: " + err;
    return rc;
  }
  return ib3d_set_mesh(c, (int64_t)m.x.size(), m.x.data(), m.y.data(), m.z.data(), (int64_t)m.e1.size(),
                       m.e1.data(), m.e2.data(), m.e3.data(), xshift, yshift, zshift, inor);
}

int ib3d_move_body_free(ib3d_ctx* c, double fx, double fy, double fz, double vel[3]) {
  if (!c) return IB3D_ERR_ARG;
  const double pi = 4.0 * std::atan(1.0);                             // subReadInput.f90:23
  const double vol = (pi * (1.0 * 1.0 * 1.0)) / 6.0;                 // :53, (pi*(1.0)**3)/6.
  const double dt = c->prm.deltat;
  const double f[3] = {fx, fy, fz};
  double v[3];
  for (int q = 0; q < 3; ++q) {
    const double init = c->motion.moving ? c->motion.vel[q] : 0.0;   // u_init = u_final (:55-57)
    v[q] = (f[q] / (vol * 1.0)) * dt + init;                           // :59-61
  }
  // xmove = u_final*deltat (:63-65); the body velocity becomes the surface velocity
  const int rc = ib3d_move_body(c, v[0] * dt, v[1] * dt, v[2] * dt, v[0], v[1], v[2]);
  if (rc) return rc;
  if (vel) for (int q = 0; q < 3; ++q) vel[q] = v[q];
  return IB3D_OK;
}

}  // extern "C"
