// A caller written the way the reference's main.cpp calls its CVT and
// rasteriser stages (main.cpp:217 through centroidalVoronoi, gcvt.h:138;
// discretization.h:66), linked against libgcvt_gb300.so instead of the
// reference's gcvt.cu / discretization.cu.  Test fixture for test_dropin.py.
//
//   dropin_main gcvt IN_SITES IN_DENSITY IN_MASK N DEPTH MAXITER OUT_LABELS
//   dropin_main raster IN_POINTS IN_WEIGHT NPOINT IN_TRIS NTRI SCALE N OUT_DENSITY
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

extern void gCVT(short *Voronoi, float *density_d, bool *mask, int size, int depth, int maxIter);
extern void discretization_d(double *points, double *weight, int num_point, int *triangle,
                             int num_tri, float *density, double scale, int n);

template <class T> static std::vector<T> slurp(const char *path, size_t count) {
  std::vector<T> v(count);
  FILE *f = std::fopen(path, "rb");
  if (!f || std::fread(v.data(), sizeof(T), count, f) != count) {
    std::fprintf(stderr, "cannot read %s\n", path);
    std::exit(2);
  }
  std::fclose(f);
  return v;
}

template <class T> static void spill(const char *path, const std::vector<T> &v) {
  FILE *f = std::fopen(path, "wb");
  if (!f || std::fwrite(v.data(), sizeof(T), v.size(), f) != v.size()) {
    std::fprintf(stderr, "cannot write %s\n", path);
    std::exit(2);
  }
  std::fclose(f);
}

int main(int argc, char **argv) {
  if (argc == 9 && !std::strcmp(argv[1], "gcvt")) {
    const int n = std::atoi(argv[5]);
    std::vector<short> voronoi = slurp<short>(argv[2], (size_t)n * n * 2);
    std::vector<float> density = slurp<float>(argv[3], (size_t)n * n);
    std::vector<unsigned char> m = slurp<unsigned char>(argv[4], (size_t)n * n);
    bool *mask = new bool[(size_t)n * n];
    for (size_t i = 0; i < m.size(); ++i) mask[i] = m[i] != 0;
    gCVT(voronoi.data(), density.data(), mask, n, std::atoi(argv[6]), std::atoi(argv[7]));
    delete[] mask;
    spill(argv[8], voronoi);
    return 0;
  }
  if (argc == 10 && !std::strcmp(argv[1], "raster")) {
    const int np = std::atoi(argv[4]), nt = std::atoi(argv[6]), n = std::atoi(argv[8]);
    std::vector<double> pts = slurp<double>(argv[2], (size_t)np * 2);
    std::vector<double> w = slurp<double>(argv[3], (size_t)np);
    std::vector<int> tri = slurp<int>(argv[5], (size_t)nt * 3);
    std::vector<float> density((size_t)n * n);
    discretization_d(pts.data(), w.data(), np, tri.data(), nt, density.data(),
                     std::atof(argv[7]), n);
    spill(argv[9], density);
    return 0;
  }
  std::fprintf(stderr, "usage: see the header of dropin_main.cpp\n");
  return 2;
}
