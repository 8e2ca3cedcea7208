// pf_paraview: the post-processor paraview.x (src/paraview.f90) with its
// voxel analysis on the GPU.
//
//   pf_paraview <input dir> <output dir> <threshold>
//
// For every step_* directory of <input dir> (in name order, as `ls` lists
// them; the part after "step_" is the step string, src/paraview.f90:65-100):
//   * reads data_extract_mult.in (Nx Ny Nz nprocs var / dims) and the
//     data_save.NNNN files 1..dims(1)*dims(2), each placed by its ist/ien
//     record (:152-172), so directories written by several ranks work too;
//   * classifies the voxels and takes |grad phi_3| on the GPU
//     (pf_analyze_fields);
//   * writes <output dir>/{phi_sq,con,var_num,phi_3,grad_phi_3,boundary}_<step>.vtk
//     (:256-296) and creates the empty step_*/var_dist the reference opens (:136);
//   * prints "<step> <precipitate voxels> <boundary voxels> <fraction>" in the
//     reference's (A, 2(I8), F6.2) after its header line (:109-110, :318).
// The reference spreads step directories over MPI ranks; here one process
// does them in order.
#include <dirent.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "pfgpu.h"

namespace {

void die(const std::string& msg) {
  fprintf(stderr, "pf_paraview: %s\n", msg.c_str());
  exit(2);
}

// one rank's record pair: "ist(3), ien(3)" and "phi(var, x, y, z), con(x, y, z)"
bool read_piece(const std::string& path, int Nx, int Ny, int Nz, int V, std::vector<double>& phi,
                std::vector<double>& con) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) return false;
  auto rec = [&](std::vector<char>& out) {
    out.clear();
    for (;;) {
      int32_t head, tail;
      if (fread(&head, 4, 1, f) != 1) return false;
      const size_t len = (size_t)(head < 0 ? -(int64_t)head : head);
      const size_t at = out.size();
      out.resize(at + len);
      if (len && fread(out.data() + at, 1, len, f) != len) return false;
      if (fread(&tail, 4, 1, f) != 1) return false;
      if (head >= 0) return true;
    }
  };
  std::vector<char> r1, r2;
  const bool ok = rec(r1) && rec(r2);
  fclose(f);
  if (!ok || r1.size() != 24) return false;
  int32_t b[6];
  memcpy(b, r1.data(), 24);
  const int x0 = b[0], y0 = b[1], z0 = b[2], x1 = b[3], y1 = b[4], z1 = b[5];
  if (x0 != 1 || x1 != Nx || y0 < 1 || y1 > Ny || z0 < 1 || z1 > Nz || y0 > y1 || z0 > z1) return false;
  const size_t ny = (size_t)(y1 - y0 + 1), nz = (size_t)(z1 - z0 + 1);
  const size_t cells = (size_t)Nx * ny * nz;
  if (r2.size() != cells * (V + 1) * sizeof(double)) return false;
  const double* p = reinterpret_cast<const double*>(r2.data());
  const double* c = p + cells * V;
  for (size_t k = 0; k < nz; ++k)
    for (size_t j = 0; j < ny; ++j) {
      const size_t src = (k * ny + j) * Nx;
      const size_t dst = ((size_t)(z0 - 1 + k) * Ny + (y0 - 1 + j)) * Nx;
      memcpy(&phi[dst * V], p + src * V, (size_t)Nx * V * sizeof(double));
      memcpy(&con[dst], c + src, (size_t)Nx * sizeof(double));
    }
  return true;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 4) {
    fprintf(stderr, "usage: pf_paraview <input dir> <output dir> <threshold>\n");
    return 1;
  }
  const std::string in_dir = argv[1], out_dir = argv[2];
  const double threshold = strtod(argv[3], nullptr);
  std::vector<std::string> steps;
  DIR* d = opendir(in_dir.c_str());
  if (!d) die("cannot list " + in_dir);
  while (dirent* e = readdir(d)) {
    const std::string name = e->d_name;
    if (name.rfind("step_", 0) != 0) continue;
    std::string s = name.substr(5);
    s = s.substr(0, s.find('_'));  // cut -d"_" -f2
    steps.push_back(s);
  }
  closedir(d);
  std::sort(steps.begin(), steps.end());
  printf("# step, precipitate_voxels,%sboundary_voxels, precipitate_fraction\n", std::string(22, ' ').c_str());
  fflush(stdout);
  const int device = getenv("PF_DEVICE") ? atoi(getenv("PF_DEVICE")) : 0;
  for (const std::string& s : steps) {
    const std::string step_dir = in_dir + "/step_" + s + "/";
    if (FILE* vd = fopen((step_dir + "var_dist").c_str(), "a")) fclose(vd);
    FILE* f = fopen((step_dir + "data_extract_mult.in").c_str(), "r");
    if (!f) die("cannot open " + step_dir + "data_extract_mult.in");
    int Nx, Ny, Nz, nprocs, V, d1 = 1, d2 = 1;
    const int got = fscanf(f, "%d %d %d %d %d %d %d", &Nx, &Ny, &Nz, &nprocs, &V, &d1, &d2);
    fclose(f);
    if (got < 5 || Nx < 1 || Ny < 1 || Nz < 1 || V < 3) die("bad data_extract_mult.in in " + step_dir);
    if (got < 7) d1 = 1, d2 = nprocs;
    const size_t n = (size_t)Nx * Ny * Nz;
    std::vector<double> phi(n * V), con(n);
    for (int fn = 1; fn <= d1 * d2; ++fn) {
      char num[16];
      snprintf(num, sizeof num, "%04d", fn);
      if (!read_piece(step_dir + "data_save." + num, Nx, Ny, Nz, V, phi, con))
        die("cannot read " + step_dir + "data_save." + num);
    }
    pf_config cfg;
    memset(&cfg, 0, sizeof cfg);
    cfg.nx = Nx; cfg.ny = Ny; cfg.nz = Nz; cfg.var = V; cfg.device = device;
    std::vector<double> phi_sq(n), phi3(n), grad(n), bnd(n);
    std::vector<int> vnum(n);
    pf_analysis_out o{phi_sq.data(), vnum.data(), phi3.data(), grad.data(), bnd.data(), nullptr};
    pf_voxel_counts cnt;
    if (pf_analyze_fields(&cfg, phi.data(), con.data(), threshold, &o, &cnt) != PF_OK)
      die(std::string("analysis of ") + step_dir + ": " + pf_last_error());
    const std::string sfx = "_" + s + ".vtk";
    struct {
      const char* name;
      const double* v;
    } reals[] = {{"phi_sq", phi_sq.data()}, {"con", con.data()}, {"phi_3", phi3.data()},
                 {"grad_phi_3", grad.data()}, {"boundary", bnd.data()}};
    for (auto& r : reals)
      if (pf_write_vtk_real((out_dir + "/" + r.name + sfx).c_str(), Nx, Ny, Nz, r.v) != PF_OK)
        die(pf_io_last_error());
    if (pf_write_vtk_int((out_dir + "/var_num" + sfx).c_str(), Nx, Ny, Nz, vnum.data()) != PF_OK)
      die(pf_io_last_error());
    printf("%s%8lld%8lld%6.2f\n", s.c_str(), cnt.precipitate_voxels, cnt.boundary_voxels, cnt.precipitate_fraction);
    fflush(stdout);
  }
  return 0;
}
