// fvc_assembly.cu -- face-coefficient assembly of the pressure-correction
// (p') system on the GPU, one thread per cell.
//
// Per cell P (original numbering) the thread gathers the vertices of P and
// of its face neighbours, then follows the reference:
//   geometry          src/Celllib.f:695-794 (cellGeom2D): vertex-average
//                     centroids, edge vectors, unit normals, centroid
//                     vectors ksi, face midpoints, normal distance ca
//   face intersection src/Celllib.f:596-655 (vectorKm2d): where the line
//                     through the centroids crosses the face -> |ksi_f|
//   coefficients      src/CellibPressure.f:476-572 (iws = 1):
//                     a_f = kf*|f|*ndd / ((n.ksi)*|ksi|), boundary faces 0,
//                     a_P = sp + sum a_f with the 1e60 pin on pin_cell
//   scatter           src/Csr.f:142-176 (CSRD) / src/EllPack.f:68-93
// Arithmetic is rounded statement by statement (no FMA contraction), so the
// coefficients equal the CPU restatement's bit for bit.  Mixed
// triangle/quad meshes use each cell's own vertex count.
#include <cstdio>

#include "fvc_internal.h"

namespace fvc {

namespace {

constexpr int kMaxSides = 4;

struct AsmArgs {
  const double *coor;   // (2, nnode)
  const int *ix;        // (ld, numel), 1-based nodes, 0 = unused slot
  int ld, numel, nshared;
  const int *nelcon;    // (nshared, numel), 1-based, -1 boundary/unused
  const int *num;       // numel, 1-based equation of each cell
  const double *kprop;  // numel
  const double *dsim;   // (2, numel)
  int pin_cell;         // 1-based, 0 none
  int int_vel;
  int matriz, unsym;
  const int *ia, *ja;   // structure (1-based)
  double *ad, *au;
};

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dvd(double a, double b) { return __ddiv_rn(a, b); }

__device__ __forceinline__ int nsides_of(const AsmArgs &a, int c) {
  int s = 0;
  while (s < a.nshared && s < a.ld && a.ix[(size_t)c * a.ld + s] > 0) ++s;
  return s;
}

// vertex-average centroid with the reference's (1/nshared)*sum scaling
__device__ __forceinline__ void centroid(const AsmArgs &a, int c, double &cx, double &cy) {
  const int ns = nsides_of(a, c);
  double sx = 0.0, sy = 0.0;
  for (int l = 0; l < ns; ++l) {
    const int no = a.ix[(size_t)c * a.ld + l] - 1;
    sx = add(sx, a.coor[2 * (size_t)no]);
    sy = add(sy, a.coor[2 * (size_t)no + 1]);
  }
  const double inv = dvd(1.0, (double)ns);
  cx = mul(inv, sx);
  cy = mul(inv, sy);
}

__global__ void assemble_pressure_kernel(AsmArgs a) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= a.numel) return;
  const int ns = nsides_of(a, c);
  double xv[kMaxSides], yv[kMaxSides];
  for (int l = 0; l < ns; ++l) {
    const int no = a.ix[(size_t)c * a.ld + l] - 1;
    xv[l] = a.coor[2 * (size_t)no];
    yv[l] = a.coor[2 * (size_t)no + 1];
  }
  double xcp, ycp;
  centroid(a, c, xcp, ycp);
  const double kP = a.kprop[c];
  const double d1P = a.dsim[2 * (size_t)c], d2P = a.dsim[2 * (size_t)c + 1];
  double coef[kMaxSides];
  int nbr[kMaxSides];
  for (int i = 0; i < a.nshared; ++i) {
    coef[i] = 0.0;
    nbr[i] = -1;
  }
  for (int i = 0; i < ns; ++i) {
    const int i2 = (i + 1) % ns;
    // edge i: nodes sn(1,i) = i, sn(2,i) = i+1
    const double ex = sub(xv[i2], xv[i]), ey = sub(yv[i2], yv[i]);
    const double meta = sqrt(add(add(0.0, mul(ex, ex)), mul(ey, ey)));
    const double ux = dvd(ex, meta), uy = dvd(ey, meta);
    const double nx = uy, ny = -ux;
    const double xm = mul(0.5, add(xv[i2], xv[i])), ym = mul(0.5, add(yv[i2], yv[i]));
    const double ca = add(mul(sub(xm, xcp), nx), mul(sub(ym, ycp), ny));
    const int vz = a.nelcon[(size_t)c * a.nshared + i];
    if (vz <= 0) continue;  // boundary (walls): a_f = 0
    const int cn = vz - 1;
    nbr[i] = cn;
    double xcn, ycn;
    centroid(a, cn, xcn, ycn);
    double kx = sub(xcn, xcp), ky = sub(ycn, ycp);
    const double mksi = sqrt(add(mul(ky, ky), add(mul(kx, kx), 0.0)));
    kx = dvd(kx, mksi);
    ky = dvd(ky, mksi);
    // vectorKm2d: intersection of the centroid line with the face line
    const double a1 = sub(ycn, ycp);
    const double b1 = sub(xcp, xcn);
    const double c1 = sub(mul(xcn, ycp), mul(xcp, ycn));
    const double a2 = sub(yv[i], yv[i2]);
    const double b2 = sub(xv[i2], xv[i]);
    const double c2 = sub(mul(xv[i], yv[i2]), mul(xv[i2], yv[i]));
    const double det = sub(mul(a1, b2), mul(a2, b1));
    const double rdet = dvd(1.0, det);
    const double m11 = mul(rdet, b2), m12 = -mul(rdet, b1);
    const double m21 = -mul(rdet, a2), m22 = mul(rdet, a1);
    const double f1 = -c1, f2 = -c2;
    const double xi1 = add(mul(m11, f1), mul(m12, f2));
    const double xi2 = add(mul(m21, f1), mul(m22, f2));
    const double kfx = sub(xi1, xcp), kfy = sub(xi2, ycp);
    const double mksif = sqrt(add(mul(kfx, kfx), mul(kfy, kfy)));
    const double alpha = dvd(mksif, mksi);
    const double oma = sub(1.0, alpha);
    const double d1n = a.dsim[2 * (size_t)cn], d2n = a.dsim[2 * (size_t)cn + 1];
    const double ddf1 = add(mul(oma, d1P), mul(alpha, d1n));
    const double ddf2 = add(mul(oma, d2P), mul(alpha, d2n));
    const double nk = add(mul(nx, kx), mul(ny, ky));
    double kf, ndd;
    if (a.int_vel == 5) {
      kf = add(mul(oma, kP), mul(alpha, a.kprop[cn]));
      ndd = mul(0.5, add(ddf1, ddf2));
    } else {
      kf = kP;
      ndd = add(mul(mul(ddf1, nx), nx), mul(mul(ddf2, ny), ny));
    }
    coef[i] = dvd(mul(mul(kf, meta), ndd), mul(nk, mksi));
    (void)ca;
  }
  double sp = 0.0;
  if (a.pin_cell == c + 1) sp = add(sp, 1.0e60);
  double ap = sp;
  for (int i = 0; i < a.nshared; ++i) ap = add(ap, coef[i]);
  const int n = a.num[c];  // 1-based row
  a.ad[n - 1] = ap;
  if (a.matriz == 4) {
    for (int j = 0; j < a.nshared; ++j)
      a.au[(size_t)(n - 1) * a.nshared + j] = (nbr[j] >= 0) ? -coef[j] : 0.0;
  } else {
    const int k0 = a.ia[n - 1] - 1, k1 = a.ia[n] - 1;
    for (int j = 0; j < a.nshared; ++j) {
      if (nbr[j] < 0) continue;
      const int l = a.num[nbr[j]];
      for (int k = k0; k < k1; ++k)
        if (a.ja[k] == l) a.au[k] = -coef[j];
    }
  }
}

}  // namespace

}  // namespace fvc

extern "C" int32_t fvc_assemble_pressure(const double *coor, int32_t nnode, const int32_t *ix,
                                         int32_t ld, int32_t numel, int32_t nshared,
                                         const int32_t *nelcon, const int32_t *num,
                                         const double *kprop, const double *dsimple,
                                         int32_t pin_cell, int32_t int_vel, int32_t matriz,
                                         int32_t unsym, const int32_t *ia, const int32_t *ja,
                                         double *ad, double *au) {
  using namespace fvc;
  if (!coor || !ix || !nelcon || !num || !kprop || !dsimple || !ad || !au || numel <= 0 ||
      nnode <= 0 || nshared < 3 || nshared > kMaxSides || ld < nshared)
    return FVC_ERR_ARG;
  if (matriz != 1 && matriz != 4) return FVC_ERR_UNSUPPORTED;
  if (matriz == 1 && (!ia || !ja)) return FVC_ERR_ARG;
  const int neq = numel;
  const size_t nad = (matriz == 1) ? (size_t)(ia[neq] - 1) : (size_t)neq * nshared;
  AsmArgs a{};
  void *bufs[12] = {nullptr};
  auto dup = [&](int slot, const void *src, size_t bytes) -> void * {
    if (cudaMalloc(&bufs[slot], bytes ? bytes : 8) != cudaSuccess) return nullptr;
    if (src && cudaMemcpy(bufs[slot], src, bytes, cudaMemcpyHostToDevice) != cudaSuccess)
      return nullptr;
    return bufs[slot];
  };
  int32_t rc = FVC_OK;
  a.coor = (const double *)dup(0, coor, sizeof(double) * 2 * (size_t)nnode);
  a.ix = (const int *)dup(1, ix, sizeof(int32_t) * (size_t)ld * numel);
  a.nelcon = (const int *)dup(2, nelcon, sizeof(int32_t) * (size_t)nshared * numel);
  a.num = (const int *)dup(3, num, sizeof(int32_t) * (size_t)numel);
  a.kprop = (const double *)dup(4, kprop, sizeof(double) * (size_t)numel);
  a.dsim = (const double *)dup(5, dsimple, sizeof(double) * 2 * (size_t)numel);
  a.ad = (double *)dup(6, nullptr, sizeof(double) * (size_t)neq);
  a.au = (double *)dup(7, nullptr, sizeof(double) * nad);
  if (matriz == 1) {
    a.ia = (const int *)dup(8, ia, sizeof(int32_t) * (size_t)(neq + 1));
    a.ja = (const int *)dup(9, ja, sizeof(int32_t) * nad);
  }
  bool ok = a.coor && a.ix && a.nelcon && a.num && a.kprop && a.dsim && a.ad && a.au &&
            (matriz == 4 || (a.ia && a.ja));
  if (ok) ok = cudaMemset(a.au, 0, sizeof(double) * nad) == cudaSuccess;
  if (ok) {
    a.ld = ld;
    a.numel = numel;
    a.nshared = nshared;
    a.pin_cell = pin_cell;
    a.int_vel = int_vel;
    a.matriz = matriz;
    a.unsym = unsym;
    assemble_pressure_kernel<<<(numel + 127) / 128, 128>>>(a);
    count_launch();
    ok = cudaDeviceSynchronize() == cudaSuccess;
  }
  if (ok)
    ok = cudaMemcpy(ad, a.ad, sizeof(double) * (size_t)neq, cudaMemcpyDeviceToHost) == cudaSuccess &&
         cudaMemcpy(au, a.au, sizeof(double) * nad, cudaMemcpyDeviceToHost) == cudaSuccess;
  if (!ok) rc = FVC_ERR_CUDA;
  for (void *p : bufs)
    if (p) cudaFree(p);
  return rc;
}
