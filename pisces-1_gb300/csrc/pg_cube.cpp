// Wavefunction files in the reference's cube formats (host code): the state
// cube of a converged vector (DVR::GetWaveFnCube, DVR::WriteCubeFile), the
// general Gaussian cube writer (WriteCubeFile) and reader (ReadCubeFile).
// Text output goes through the same printf formats as the reference, so a
// file written here is byte-identical to the reference's for the same data.
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "pg_common.cuh"

namespace {

// src/constants.h:18-19
constexpr double kBohr2Angs = 0.52917720859;
const double kAngs2Bohr = 1 / kBohr2Angs;

// van der Waals radius (Angstrom) written beside each atom for cube
// integration programs (src/WriteCubeFile.cpp:44-53, src/DVR.cpp:1984-1993)
double vdw_radius(int z) {
  switch (z) {
    case 1: return 1.20;
    case 6: return 1.70;
    case 7: return 1.55;
    case 8: return 1.52;
    default: return 0.0;
  }
}

void write_atoms(FILE* f, int natoms, const int* Z, const double* pos_angstrom) {
  for (int k = 0; k < natoms; ++k) {
    const double* r = pos_angstrom + 3 * k;
    fprintf(f, "   %i %11.6f  %11.6f  %11.6f  %11.6f\n", Z[k], vdw_radius(Z[k]) * kAngs2Bohr, r[0] * kAngs2Bohr,
            r[1] * kAngs2Bohr, r[2] * kAngs2Bohr);
  }
}

// values with z fastest, six per line, each z run ending its line
void write_values(FILE* f, int nx, int ny, int nz, const double* v) {
  const int per_line = 6;
  long c = 0;
  for (int ix = 0; ix < nx; ++ix)
    for (int iy = 0; iy < ny; ++iy) {
      int k = 1;
      for (int iz = 0; iz < nz; ++iz) {
        fprintf(f, "%13.6e ", v[c++]);
        if (k % per_line == 0) fprintf(f, "\n");
        ++k;
      }
      if (nz % per_line != 0) fprintf(f, "\n");
    }
}

// Volume element of the equidistant DVR grid, (x_{n-1} - x_0) / (n - 1) per
// axis.  The reference takes all three extents at index nz-1
// (src/DVR.cpp:1924, 2051), which equals this on cubic grids and reads past
// the x and y points on others; the per-axis extents are used here.
double volume_element(const pg_grid* g) {
  const double ex = g->x[0][g->n[0] - 1] - g->x[0][0], ey = g->x[1][g->n[1] - 1] - g->x[1][0],
               ez = g->x[2][g->n[2] - 1] - g->x[2][0];
  return ez * ey * ex / double((long)(g->n[0] - 1) * (g->n[1] - 1) * (g->n[2] - 1));
}

}  // namespace

extern "C" pg_status pg_state_cube(const pg_grid* g, const double* wf, double* cube) {
  PG_ARG(g && wf && cube, "pg_state_cube: null argument");
  PG_ARG(g->n[0] > 1 && g->n[1] > 1 && g->n[2] > 1, "pg_state_cube: every axis needs two points");
  const int nx = g->n[0], ny = g->n[1], nz = g->n[2];
  const double oosqrdv = 1.0 / sqrt(volume_element(g));
  double* c = cube;
  for (int ix = 0; ix < nx; ++ix)
    for (int iy = 0; iy < ny; ++iy)
      for (int iz = 0; iz < nz; ++iz) *c++ = wf[ix + (long)nx * (iy + (long)ny * iz)] * oosqrdv;
  return PG_OK;
}

extern "C" pg_status pg_write_state_cube(const pg_grid* g, const double* wf, int iwf, const char* path, int natoms,
                                         const int* Z, const double* pos_angstrom, int cubeflag, double* integral) {
  PG_ARG(g && wf && path && natoms >= 0 && (natoms == 0 || (Z && pos_angstrom)), "pg_write_state_cube: bad arguments");
  PG_ARG(g->n[0] > 1 && g->n[1] > 1 && g->n[2] > 1, "pg_write_state_cube: every axis needs two points");
  const int nx = g->n[0], ny = g->n[1], nz = g->n[2];
  const double* xg = g->x[0].data();
  const double* yg = g->x[1].data();
  const double* zg = g->x[2].data();
  const double dV = volume_element(g);
  const double oosqrdv = 1.0 / sqrt(dV);
  FILE* f = fopen(path, "w+");
  if (!f) {
    pg::set_error("pg_write_state_cube: cannot open %s", path);
    return PG_BAD_ARG;
  }
  double intr = 0.0;
  if (cubeflag == 1) {
    // gOpenMol text grid (src/DVR.cpp:1944-1960): z slowest in the header,
    // extents in Angstrom, one value per line with x fastest
    fprintf(f, "3 3\n%i %i %i\n", nz, ny, nx);
    const double B2A = kBohr2Angs;
    fprintf(f, "%13.6e %13.6e    %13.6e %13.6e    %13.6e %13.6e\n", zg[0] * B2A, zg[nz - 1] * B2A, yg[0] * B2A,
            yg[ny - 1] * B2A, xg[0] * B2A, xg[nx - 1] * B2A);
    for (int iz = 0; iz < nz; ++iz)
      for (int iy = 0; iy < ny; ++iy)
        for (int ix = 0; ix < nx; ++ix) {
          const double rho = wf[ix + (long)nx * (iy + (long)ny * iz)] * oosqrdv;
          fprintf(f, "%13.6e\n", rho);
          intr += rho * rho;
        }
  } else {
    // Gaussian cube of an orbital (src/DVR.cpp:1961-2016): negative atom
    // count, then the orbital line "1 iwf"
    const double nought = 0.0;
    fprintf(f, " 5 0\n");
    fprintf(f, " 0.01 0.001 0.0001 0.00001 0.000001\n");
    fprintf(f, "%5i  %11.6f  %11.6f  %11.6f\n", -natoms, xg[0], yg[0], zg[0]);
    fprintf(f, "%5i  %11.6f  %11.6f  %11.6f\n", nx, xg[1] - xg[0], nought, nought);
    fprintf(f, "%5i  %11.6f  %11.6f  %11.6f\n", ny, nought, yg[1] - yg[0], nought);
    fprintf(f, "%5i  %11.6f  %11.6f  %11.6f\n", nz, nought, nought, zg[1] - zg[0]);
    write_atoms(f, natoms, Z, pos_angstrom);
    fprintf(f, "   1  %5i \n", iwf);
    const int per_line = 6;
    for (int ix = 0; ix < nx; ++ix)
      for (int iy = 0; iy < ny; ++iy) {
        int k = 1;
        for (int iz = 0; iz < nz; ++iz) {
          const double rho = wf[ix + (long)nx * (iy + (long)ny * iz)] * oosqrdv;
          fprintf(f, "%13.6e ", rho);
          if (k % per_line == 0) fprintf(f, "\n");
          ++k;
          intr += rho * rho;
        }
        if (nz % per_line != 0) fprintf(f, "\n");
      }
  }
  const bool bad = ferror(f) != 0;
  fclose(f);
  if (bad) {
    pg::set_error("pg_write_state_cube: write to %s failed", path);
    return PG_BAD_ARG;
  }
  if (integral) *integral = intr * dV;
  return PG_OK;
}

extern "C" pg_status pg_write_cube(const char* path, int natoms, const int* Z, const double* pos_angstrom,
                                   const int npts[3], const double x0[3], const double dx[3], const double* cube) {
  PG_ARG(path && npts && x0 && dx && cube && natoms >= 0 && (natoms == 0 || (Z && pos_angstrom)),
         "pg_write_cube: bad arguments");
  PG_ARG(npts[0] > 0 && npts[1] > 0 && npts[2] > 0, "pg_write_cube: empty grid");
  FILE* f = fopen(path, "w+");
  if (!f) {
    pg::set_error("pg_write_cube: cannot open %s", path);
    return PG_BAD_ARG;
  }
  // src/WriteCubeFile.cpp:31-75
  const double nought = 0.0;
  fprintf(f, " 5 0  (these 2 lines are for cubeint)\n");
  fprintf(f, " 0.01 0.001 0.0001 0.00001 0.000001\n");
  fprintf(f, "%5i  %11.6f  %11.6f  %11.6f\n", natoms, x0[0], x0[1], x0[2]);
  fprintf(f, "%5i  %11.6f  %11.6f  %11.6f\n", npts[0], dx[0], nought, nought);
  fprintf(f, "%5i  %11.6f  %11.6f  %11.6f\n", npts[1], nought, dx[1], nought);
  fprintf(f, "%5i  %11.6f  %11.6f  %11.6f\n", npts[2], nought, nought, dx[2]);
  write_atoms(f, natoms, Z, pos_angstrom);
  write_values(f, npts[0], npts[1], npts[2], cube);
  const bool bad = ferror(f) != 0;
  fclose(f);
  if (bad) {
    pg::set_error("pg_write_cube: write to %s failed", path);
    return PG_BAD_ARG;
  }
  return PG_OK;
}

extern "C" pg_status pg_read_cube(const char* path, int npts[3], double x0[3], double dx[3], int* natoms,
                                  double* cube, long capacity) {
  PG_ARG(path && npts && x0 && dx, "pg_read_cube: null argument");
  FILE* f = fopen(path, "r");
  if (!f) {
    pg::set_error("pg_read_cube: cannot open %s", path);
    return PG_BAD_ARG;
  }
  auto next_line = [&](std::string& s) -> bool {
    s.clear();
    int c;
    while ((c = fgetc(f)) != EOF && c != '\n') s.push_back((char)c);
    return !(c == EOF && s.empty());
  };
  auto fail = [&](const char* what) {
    fclose(f);
    pg::set_error("pg_read_cube: %s: %s", path, what);
    return PG_BAD_ARG;
  };
  std::string s;
  // two comment lines, then the atom count and origin, then one line per axis
  // (src/ReadCubeFile.cpp:33-62); only cartesian grids
  if (!next_line(s) || !next_line(s)) return fail("missing comment lines");
  int nnuc = 0;
  if (!next_line(s) || sscanf(s.c_str(), "%i %lf %lf %lf", &nnuc, x0, x0 + 1, x0 + 2) != 4)
    return fail("bad atom-count line");
  for (int a = 0; a < 3; ++a) {
    double v[3];
    if (!next_line(s) || sscanf(s.c_str(), "%i %lf %lf %lf", &npts[a], v, v + 1, v + 2) != 4)
      return fail("bad axis line");
    for (int b = 0; b < 3; ++b)
      if (b != a && v[b] != 0) return fail("only cartesian grids");
    dx[a] = v[a];
    if (npts[a] <= 0) return fail("non-positive point count");
  }
  if (natoms) *natoms = nnuc;
  // atom lines; a negative count marks an orbital cube, whose atom lines are
  // followed by the orbital-index line (the reference's reader expects a
  // positive count)
  const int skip = nnuc >= 0 ? nnuc : -nnuc + 1;
  for (int i = 0; i < skip; ++i)
    if (!next_line(s)) return fail("missing atom lines");
  const long total = (long)npts[0] * npts[1] * npts[2];
  if (!cube) {
    fclose(f);
    return PG_OK;
  }
  if (capacity < total) {
    fclose(f);
    pg::set_error("pg_read_cube: %s holds %ld values, the buffer %ld", path, total, capacity);
    return PG_BAD_ARG;
  }
  for (long i = 0; i < total; ++i)
    if (fscanf(f, "%lf", &cube[i]) != 1) return fail("fewer values than the grid has points");
  fclose(f);
  return PG_OK;
}
