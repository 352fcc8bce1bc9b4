// rfgpu_abi_smoke.cpp - a C++ caller of include/rfgpu.h, built with g++ and
// linked against librfgpu.so, standing in for the Fortran host of the
// reference: it registers one region from arrays in the Fortran memory image
// and drives the time-step loop the way rocflu/RFLU_TimeStepping.F90 and
// libfloflu/RungeKuttaMP.F90 would once their stage loop calls the C ABI
// (rfgpu_dt, then rfgpu_stage for every RK stage, rfgpu_status, rfgpu_download,
// rfgpu_region_destroy).
//
// The layout expectations of the shared structs (every field's offset and
// each struct's size, computed from the BIND(C) derived types of the Fortran
// binding module) come from the generated header named by RFGPU_LAYOUT_H and
// are checked at compile time.
//
// Usage: rfgpu_abi_smoke <dir>.  <dir>/meta.txt holds, whitespace separated:
//   nCells nFaces nMembs nPatches spaceDiscr spaceOrder reconst rkScheme
//   precision venkatGuard refCp refGamma gvCp gvMol epsentr dissFact cfl nSteps
//   then per patch: bcType spaceOrder bcOptType nBFaces
// and the arrays are raw little-endian files: f2c.i32 (2,nFaces), fn.f64
// (4,nFaces), fc.f64 (3,nFaces), cofg.f64 (3,nCells), vol.f64, c2csoff.i32
// (nCells+1), c2csmem.i32, xyzmoms.f64 (10,nCells), cv.f64 (5,nCells), dv.f64
// (3,nCells), per patch pK_bf2c.i32, pK_fn.f64, pK_fc.f64.  It writes
// out_cv.f64, out_dv.f64 and out.txt ("status time") and exits 0 on success.
#include "rfgpu.h"

#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

#ifdef RFGPU_LAYOUT_H
#include RFGPU_LAYOUT_H
#endif

namespace {

template <typename T>
std::vector<T> read_raw(const std::string &path, size_t n) {
  std::vector<T> v(n);
  FILE *f = std::fopen(path.c_str(), "rb");
  if (!f || std::fread(v.data(), sizeof(T), n, f) != n) {
    std::fprintf(stderr, "cannot read %s\n", path.c_str());
    std::exit(2);
  }
  std::fclose(f);
  return v;
}

template <typename T>
void write_raw(const std::string &path, const std::vector<T> &v) {
  FILE *f = std::fopen(path.c_str(), "wb");
  if (!f || std::fwrite(v.data(), sizeof(T), v.size(), f) != v.size()) {
    std::fprintf(stderr, "cannot write %s\n", path.c_str());
    std::exit(2);
  }
  std::fclose(f);
}

int fail(const char *what, int rc) {
  std::fprintf(stderr, "%s returned %d\n", what, rc);
  return 1;
}

}  // namespace

int main(int argc, char **argv) {
  if (argc != 2) {
    std::fprintf(stderr, "usage: %s <dir>\n", argv[0]);
    return 2;
  }
  const std::string dir = argv[1];
  std::ifstream meta(dir + "/meta.txt");
  int nCells, nFaces, nMembs, nPatches, spaceDiscr, spaceOrder, reconst, rkScheme, precision,
      venkatGuard, nSteps;
  double refCp, refGamma, gvCp, gvMol, epsentr, dissFact, cfl;
  meta >> nCells >> nFaces >> nMembs >> nPatches >> spaceDiscr >> spaceOrder >> reconst >>
      rkScheme >> precision >> venkatGuard >> refCp >> refGamma >> gvCp >> gvMol >> epsentr >>
      dissFact >> cfl >> nSteps;
  if (!meta) {
    std::fprintf(stderr, "bad meta.txt\n");
    return 2;
  }
  const size_t N = (size_t)nCells, F = (size_t)nFaces;
  auto f2c = read_raw<int>(dir + "/f2c.i32", 2 * F);
  auto fn = read_raw<double>(dir + "/fn.f64", 4 * F);
  auto fc = read_raw<double>(dir + "/fc.f64", 3 * F);
  auto cofg = read_raw<double>(dir + "/cofg.f64", 3 * N);
  auto vol = read_raw<double>(dir + "/vol.f64", N);
  auto off = read_raw<int>(dir + "/c2csoff.i32", N + 1);
  auto mem = read_raw<int>(dir + "/c2csmem.i32", (size_t)nMembs);
  auto moms = read_raw<double>(dir + "/xyzmoms.f64", 10 * N);
  auto cv = read_raw<double>(dir + "/cv.f64", 5 * N);
  auto dv = read_raw<double>(dir + "/dv.f64", 3 * N);
  std::vector<rfgpu_patch_t> patches((size_t)nPatches);
  std::vector<std::vector<int>> pb2c((size_t)nPatches);
  std::vector<std::vector<double>> pfn((size_t)nPatches), pfc((size_t)nPatches);
  for (int ip = 0; ip < nPatches; ++ip) {
    rfgpu_patch_t &p = patches[(size_t)ip];
    meta >> p.bcType >> p.spaceOrder >> p.bcOptType >> p.nBFaces;
    const std::string k = dir + "/p" + std::to_string(ip);
    pb2c[(size_t)ip] = read_raw<int>(k + "_bf2c.i32", (size_t)p.nBFaces);
    pfn[(size_t)ip] = read_raw<double>(k + "_fn.f64", 4 * (size_t)p.nBFaces);
    pfc[(size_t)ip] = read_raw<double>(k + "_fc.f64", 3 * (size_t)p.nBFaces);
    p.bf2c = pb2c[(size_t)ip].data();
    p.fn = pfn[(size_t)ip].data();
    p.fc = pfc[(size_t)ip].data();
    p.vals = nullptr;   // slip walls and supersonic outflow need no patch values
    p.distrib = 0;
    p.nData = 0;
    p.bcOptFixed = 0;
    p.nBFacesTot = 0;   // one region: no faces on virtual cells
  }
  rfgpu_region_desc_t d{};
  d.nCells = nCells;
  d.nFaces = nFaces;
  d.f2cLd = 2;
  d.f2c = f2c.data();
  d.fn = fn.data();
  d.fc = fc.data();
  d.cofg = cofg.data();
  d.vol = vol.data();
  d.c2csOffsets = off.data();
  d.c2csMembers = mem.data();
  d.xyzMoms = moms.data();
  d.nPatches = nPatches;
  d.patches = patches.data();
  d.cv = cv.data();
  d.dv = dv.data();
  d.gasModel = RFGPU_GAS_MODEL_TCPERF;
  d.flowModel = RFGPU_FLOW_EULER;
  d.spaceDiscr = spaceDiscr;
  d.spaceOrder = spaceOrder;
  d.reconst = reconst;
  d.rkScheme = rkScheme;
  d.refCp = refCp;
  d.refGamma = refGamma;
  d.gvCp = gvCp;
  d.gvMol = gvMol;
  d.epsentr = epsentr;
  d.dissFact = dissFact;
  d.precision = precision;
  d.venkatGuard = venkatGuard;
  d.cellOrder = RFGPU_ORDER_LOCALITY;
  d.ausmSigma = 1.0;
  d.ausmKp = 0.25;
  d.ausmKu = 0.75;
  d.ausmMInf = 0.1;
  d.nCellsTot = 0;
  d.iRegionGlobal = 1;
  d.nBorders = 0;
  d.borders = nullptr;

  rfgpu_region_t h = nullptr;
  int rc = rfgpu_region_create(&d, &h);
  if (rc != RFGPU_OK) return fail("rfgpu_region_create", rc);
  // RFLU_TimeStepping: the first step takes dtImposed, here the CFL step of
  // the initial state (asked for with currentTime > 1e-8)
  double dtImposed = 0.0;
  rc = rfgpu_dt(h, cfl, 1.0, 0.0, 1.0, &dtImposed);
  if (rc != RFGPU_OK) return fail("rfgpu_dt", rc);
  const int nrk = rkScheme == RFGPU_RK_SCHEME_4_CLASSICAL ? 4 : rkScheme == RFGPU_RK_SCHEME_3_WRAY ? 3 : 1;
  double t = 0.0;
  for (int step = 0; step < nSteps; ++step) {
    double dtMin = 0.0;
    rc = rfgpu_dt(h, cfl, dtImposed, 0.0, t, &dtMin);
    if (rc != RFGPU_OK) return fail("rfgpu_dt", rc);
    for (int is = 1; is <= nrk; ++is) {
      rc = rfgpu_stage(h, is, dtMin);
      if (rc != RFGPU_OK) return fail("rfgpu_stage", rc);
    }
    t += dtMin;
  }
  int flags = 0;
  rc = rfgpu_status(h, &flags);
  if (rc != RFGPU_OK) return fail("rfgpu_status", rc);
  std::vector<double> cvo(5 * N), dvo(3 * N);
  rc = rfgpu_download(h, cvo.data(), dvo.data());
  if (rc != RFGPU_OK) return fail("rfgpu_download", rc);
  rc = rfgpu_region_destroy(h);
  if (rc != RFGPU_OK) return fail("rfgpu_region_destroy", rc);
  write_raw(dir + "/out_cv.f64", cvo);
  write_raw(dir + "/out_dv.f64", dvo);
  FILE *o = std::fopen((dir + "/out.txt").c_str(), "w");
  if (!o) return 2;
  std::fprintf(o, "%d %.17g\n", flags, t);
  std::fclose(o);
  return 0;
}
