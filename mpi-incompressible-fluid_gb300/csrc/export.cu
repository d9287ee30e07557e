// VTK and DAT writers for one rank (host side). The byte layouts are the
// reference's (src/VTKDatExport.cpp): the files can be compared byte for byte
// and read by the reference's post-processing. The arithmetic is done in the
// context's Real type (double for an FP64 context, float for a mixed one, as
// the reference computes with its own Real) and in the reference's operation
// order, on values fetched from the device in small boxes.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <vector>

#include "../../include/mifgpu.h"
#include "export.cuh"

namespace mifgpu {

namespace {

// The index bookkeeping of the reference's COMPUTE_INDEXING for one rank
// (src/VTKDatExport.cpp:97-121 with Py = Pz = 1, src/Constants.cpp:58-101):
// every axis writes Ng points from local index s, s = 1 only on a periodic x
// axis (on one rank the y and z neighbours are -1, so those start at 0 even
// when periodic).
template <typename R>
struct Layout {
  long N[3];       // points written per axis
  int s[3];        // first local index
  long gs[3];      // first global index (base + s)
  R mn[3], d[3];   // min_*_global, dx/dy/dz
  int base[3];
  explicit Layout(const ExportSource &src) {
    const Geometry &g = src.g;
    for (int a = 0; a < 3; ++a) {
      N[a] = g.n_global[a];
      s[a] = (a == 0 && g.periodic[0]) ? 1 : 0;
      base[a] = g.base[a];
      gs[a] = base[a] + s[a];
      mn[a] = R(g.origin[a]);
      d[a] = R(src.size[a]) / R(g.n_global[a] - 1);  // Constants: size / (Ng - 1) in Real
    }
  }
  R coord(int a, long idx) const { return mn[a] + R(base[a] + idx) * d[a]; }
};

// pos_to_index of src/VTKDatExport.cpp:50-56: the index of the closest
// pressure plane at or below pos and its weight, returned through a float.
template <typename R>
void pos_to_index(R pos, R mn, R delta, long &index, R &weight) {
  const R offset = pos - mn;
  const R fi = offset / delta;
  const R i1 = std::floor(fi);
  const R imp = R(1.0) - (fi - i1);
  index = (long)i1;
  weight = R((float)imp);
}

// Values of one field on an index box (x fastest).
struct Block {
  long lo[3] = {0, 0, 0}, n[3] = {0, 0, 0};
  std::vector<double> v;
  bool get(long i, long j, long k, double &out) const {
    const long a = i - lo[0], b = j - lo[1], c = k - lo[2];
    if (a < 0 || b < 0 || c < 0 || a >= n[0] || b >= n[1] || c >= n[2]) return false;
    out = v[(size_t)(a + n[0] * (b + n[1] * c))];
    return true;
  }
};

// One field on the index box the writers read. An index is resolved the way
// the reference's tensors resolve it, through the flat offset
// i + Ex (j + Ey k) of the field's storage (include/Tensor.h:137-140): on a
// periodic x axis the writers read u one past the end of a row
// (src/VTKDatExport.cpp:155, 391), which is the first element of the next
// row, and likewise v one row past the end of a plane. `wrap` holds the
// points such reads land on. Reads outside the storage give 0 (they only
// occur multiplied by a zero weight, or past the last plane, where the
// reference reads beyond its allocation).
struct Box {
  long ext[3] = {0, 0, 0};
  Block main, wrap;
  double at(long i, long j, long k) const {
    const long f = i + ext[0] * (j + ext[1] * k);
    if (f < 0 || f >= ext[0] * ext[1] * ext[2]) return 0.0;
    const long fi = f % ext[0], fj = (f / ext[0]) % ext[1], fk = f / (ext[0] * ext[1]);
    double x = 0.0;
    if (main.get(fi, fj, fk, x) || wrap.get(fi, fj, fk, x)) return x;
    return 0.0;
  }
};

// Extent of field id (0..2 velocity, 9 pressure) along axis d.
int field_ext(const Geometry &g, int id, int d) { return id < 3 ? g.ext(id, d) : g.E[d]; }

int fetch_block(const ExportSource &src, int id, Block &blk) {
  blk.v.assign((size_t)(blk.n[0] * blk.n[1] * blk.n[2]), 0.0);
  if (blk.v.empty()) return MIFGPU_OK;
  const int lo[3] = {(int)blk.lo[0], (int)blk.lo[1], (int)blk.lo[2]};
  const int n[3] = {(int)blk.n[0], (int)blk.n[1], (int)blk.n[2]};
  return src.fetch(id, lo, n, blk.v.data());
}

// Fetches field id for reads on [lo, hi): the box clipped to the field's
// extents, and the bounding box of the in-storage points that reads past
// the x or y extent resolve to.
int fetch_box(const ExportSource &src, int id, const long lo[3], const long hi[3], Box &b) {
  for (int d = 0; d < 3; ++d) {
    b.ext[d] = field_ext(src.g, id, d);
    b.main.lo[d] = std::max(lo[d], 0L);
    b.main.n[d] = std::max(std::min(hi[d], b.ext[d]) - b.main.lo[d], 0L);
  }
  long wlo[3] = {b.ext[0], b.ext[1], b.ext[2]}, whi[3] = {0, 0, 0};
  auto note = [&](long i, long j, long k) {
    const long f = i + b.ext[0] * (j + b.ext[1] * k);
    if (f < 0 || f >= b.ext[0] * b.ext[1] * b.ext[2]) return;
    const long q[3] = {f % b.ext[0], (f / b.ext[0]) % b.ext[1], f / (b.ext[0] * b.ext[1])};
    for (int d = 0; d < 3; ++d) {
      wlo[d] = std::min(wlo[d], q[d]);
      whi[d] = std::max(whi[d], q[d] + 1);
    }
  };
  const long k0 = std::max(lo[2], 0L), j0 = std::max(lo[1], 0L);
  for (long k = k0; k < hi[2]; ++k) {
    for (long j = j0; j < hi[1]; ++j) {
      const long i0 = j < b.ext[1] ? std::max(lo[0], b.ext[0]) : std::max(lo[0], 0L);
      for (long i = i0; i < hi[0]; ++i) note(i, j, k);
    }
  }
  for (int d = 0; d < 3; ++d) {
    b.wrap.lo[d] = wlo[d];
    b.wrap.n[d] = std::max(whi[d] - wlo[d], 0L);
  }
  if (int rc = fetch_block(src, id, b.main)) return rc;
  return fetch_block(src, id, b.wrap);
}

// The four fields on one index box (velocity set 0 and the pressure).
struct State {
  Box f[4];  // u, v, w, p
  int load(const ExportSource &src, const long lo[3], const long hi[3]) {
    const int ids[4] = {0, 1, 2, 9};
    for (int q = 0; q < 4; ++q)
      if (int rc = fetch_box(src, ids[q], lo, hi, f[q])) return rc;
    return MIFGPU_OK;
  }
};

template <typename R>
R big_endian(R x) {
  if constexpr (sizeof(R) == 8) {
    uint64_t u;
    std::memcpy(&u, &x, 8);
    u = __builtin_bswap64(u);
    std::memcpy(&x, &u, 8);
  } else {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    u = __builtin_bswap32(u);
    std::memcpy(&x, &u, 4);
  }
  return x;
}

template <typename R>
int vtk_planes(const ExportSource &src, const char *filename, std::string &err) {
  const Layout<R> L(src);
  std::vector<R> xyz, pu, pv, pw, pp;
  auto put = [&](const State &S, long i, long j, long k) {
    xyz.push_back(L.coord(0, i));
    xyz.push_back(L.coord(1, j));
    xyz.push_back(L.coord(2, k));
    pu.push_back((R(S.f[0].at(i, j, k)) + R(S.f[0].at(i + 1, j, k))) / 2);
    pv.push_back((R(S.f[1].at(i, j, k)) + R(S.f[1].at(i, j + 1, k))) / 2);
    pw.push_back((R(S.f[2].at(i, j, k)) + R(S.f[2].at(i, j, k + 1))) / 2);
    pp.push_back(R(S.f[3].at(i, j, k)));
  };
  const long ei = L.s[0] + L.N[0], ej = L.s[1] + L.N[1], ek = L.s[2] + L.N[2];
  // z = 0 plane (written first), then x = 0, then y = 0 (src/VTKDatExport.cpp:161-204)
  long kg, ig, jg;
  R w;
  pos_to_index<R>(R(0.0), L.mn[2], L.d[2], kg, w);
  if (kg >= L.gs[2] && kg < L.gs[2] + L.N[2]) {
    const long k = kg - L.gs[2] + L.s[2];
    const long lo[3] = {L.s[0], L.s[1], k}, hi[3] = {ei + 1, ej + 1, k + 2};
    State S;
    if (int rc = S.load(src, lo, hi)) return rc;
    for (long i = L.s[0]; i < ei; ++i)
      for (long j = L.s[1]; j < ej; ++j) put(S, i, j, k);
  }
  pos_to_index<R>(R(0.0), L.mn[0], L.d[0], ig, w);
  if (!(ig >= L.gs[0] && ig < L.gs[0] + L.N[0])) {
    err = "write_vtk: the plane x = 0 is outside the domain";
    return MIFGPU_EINVAL;
  }
  {
    const long i = ig - L.gs[0] + L.s[0];
    const long lo[3] = {i, L.s[1], L.s[2]}, hi[3] = {i + 2, ej + 1, ek + 1};
    State S;
    if (int rc = S.load(src, lo, hi)) return rc;
    for (long j = L.s[1]; j < ej; ++j)
      for (long k = L.s[2]; k < ek; ++k) put(S, i, j, k);
  }
  pos_to_index<R>(R(0.0), L.mn[1], L.d[1], jg, w);
  if (jg >= L.gs[1] && jg < L.gs[1] + L.N[1]) {
    const long j = jg - L.gs[1] + L.s[1];
    const long lo[3] = {L.s[0], j, L.s[2]}, hi[3] = {ei + 1, j + 2, ek + 1};
    State S;
    if (int rc = S.load(src, lo, hi)) return rc;
    for (long i = L.s[0]; i < ei; ++i)
      for (long k = L.s[2]; k < ek; ++k) put(S, i, j, k);
  }
  const int n = (int)pu.size();
  for (auto *vec : {&xyz, &pu, &pv, &pw, &pp})
    for (R &x : *vec) x = big_endian(x);
  FILE *f = std::fopen(filename, "wb");
  if (!f) {
    err = std::string("write_vtk: cannot open ") + filename;
    return MIFGPU_EINVAL;
  }
  const char *ty = sizeof(R) == 8 ? "double" : "float";
  char buf[256];
  int len = std::snprintf(buf, sizeof(buf),
                          "# vtk DataFile Version 2.0\nvtk output\nBINARY\nDATASET UNSTRUCTURED_GRID \nPOINTS %d %s\n",
                          n, ty);
  std::fwrite(buf, 1, (size_t)len, f);
  std::fwrite(xyz.data(), sizeof(R), xyz.size(), f);
  len = std::snprintf(buf, sizeof(buf), "\nPOINT_DATA %d\nSCALARS u %s 1\nLOOKUP_TABLE default\n", n, ty);
  std::fwrite(buf, 1, (size_t)len, f);
  std::fwrite(pu.data(), sizeof(R), pu.size(), f);
  const char *names[3] = {"v", "w", "p"};
  const std::vector<R> *cols[3] = {&pv, &pw, &pp};
  for (int q = 0; q < 3; ++q) {
    len = std::snprintf(buf, sizeof(buf), "\nSCALARS %s %s 1\nLOOKUP_TABLE default\n", names[q], ty);
    std::fwrite(buf, 1, (size_t)len, f);
    std::fwrite(cols[q]->data(), sizeof(R), cols[q]->size(), f);
  }
  std::fclose(f);
  return MIFGPU_OK;
}

template <typename R>
int dat_line(const ExportSource &src, const char *filename, int direction, R x, R y, R z, std::string &err) {
  if (direction < 0 || direction > 2) {
    err = "write_dat: direction must be 0, 1 or 2";
    return MIFGPU_EINVAL;
  }
  const Layout<R> L(src);
  long ig, jg, kg;
  R wi, wj, wk;
  pos_to_index<R>(x, L.mn[0], L.d[0], ig, wi);
  pos_to_index<R>(y, L.mn[1], L.d[1], jg, wj);
  pos_to_index<R>(z, L.mn[2], L.d[2], kg, wk);
  const R tol = R(1e-6);
  auto ok = [&](R w) { return std::abs(w - R(1.0)) < tol || std::abs(w - R(0.5)) < tol; };
  if (!ok(wi) || !ok(wj) || !ok(wk)) {
    err = "write_dat: the line must pass through pressure planes or midway between them";
    return MIFGPU_EINVAL;
  }
  const bool ax = std::abs(wi - R(1.0)) < tol, ay = std::abs(wj - R(1.0)) < tol, az = std::abs(wk - R(1.0)) < tol;
  const long ei = L.s[0] + L.N[0], ej = L.s[1] + L.N[1], ek = L.s[2] + L.N[2];
  auto in = [&](int a, long gidx) { return gidx >= L.gs[a] && gidx < L.gs[a] + L.N[a]; };
  std::vector<R> cs, du, dv, dw, dp;
  const long i = ig - L.gs[0] + L.s[0], j = jg - L.gs[1] + L.s[1], k = kg - L.gs[2] + L.s[2];
  State S;
  // The weighted sums of src/VTKDatExport.cpp:390-509, term for term (the
  // y and z lines read v where u is meant in the midway-x case; kept).
  if (direction == 0 && in(1, jg) && in(2, kg)) {
    const long lo[3] = {L.s[0], j, k}, hi[3] = {ei + 1, j + 2, k + 2};
    if (int rc = S.load(src, lo, hi)) return rc;
    auto U = [&](long a, long b, long c) { return R(S.f[0].at(a, b, c)); };
    auto V = [&](long a, long b, long c) { return R(S.f[1].at(a, b, c)); };
    auto W = [&](long a, long b, long c) { return R(S.f[2].at(a, b, c)); };
    auto P = [&](long a, long b, long c) { return R(S.f[3].at(a, b, c)); };
    for (long ii = L.s[0]; ii < ei; ++ii) {
      cs.push_back(L.coord(0, ii));
      du.push_back(wj * wk * (U(ii, j, k) + U(ii + 1, j, k)) / 2 +
                   (1 - wj) * wk * (U(ii, j + 1, k) + U(ii + 1, j + 1, k)) / 2 +
                   wj * (1 - wk) * (U(ii, j, k + 1) + U(ii + 1, j, k + 1)) / 2 +
                   (1 - wj) * (1 - wk) * (U(ii, j + 1, k + 1) + U(ii + 1, j + 1, k + 1)) / 2);
      if (ay)
        dv.push_back(wk * (V(ii, j, k) + V(ii, j + 1, k)) / 2 + (1 - wk) * (V(ii, j, k + 1) + V(ii, j + 1, k + 1)) / 2);
      else
        dv.push_back(wk * V(ii, j + 1, k) + (1 - wk) * V(ii, j + 1, k + 1));
      if (az)
        dw.push_back(wj * (W(ii, j, k) + W(ii, j, k + 1)) / 2 + (1 - wj) * (W(ii, j + 1, k) + W(ii, j + 1, k + 1)) / 2);
      else
        dw.push_back(wj * W(ii, j, k + 1) + (1 - wj) * W(ii, j + 1, k + 1));
      dp.push_back(wj * wk * P(ii, j, k) + (1 - wj) * wk * P(ii, j + 1, k) + wj * (1 - wk) * P(ii, j, k + 1) +
                   (1 - wj) * (1 - wk) * P(ii, j + 1, k + 1));
    }
  } else if (direction == 1 && in(0, ig) && in(2, kg)) {
    const long lo[3] = {i, L.s[1], k}, hi[3] = {i + 2, ej + 1, k + 2};
    if (int rc = S.load(src, lo, hi)) return rc;
    auto U = [&](long a, long b, long c) { return R(S.f[0].at(a, b, c)); };
    auto V = [&](long a, long b, long c) { return R(S.f[1].at(a, b, c)); };
    auto W = [&](long a, long b, long c) { return R(S.f[2].at(a, b, c)); };
    auto P = [&](long a, long b, long c) { return R(S.f[3].at(a, b, c)); };
    for (long jj = L.s[1]; jj < ej; ++jj) {
      cs.push_back(L.coord(1, jj));
      if (ax)
        du.push_back(wk * (U(i, jj, k) + U(i + 1, jj, k)) / 2 + (1 - wk) * (U(i, jj, k + 1) + U(i + 1, jj, k + 1)) / 2);
      else
        du.push_back(wk * U(i + 1, jj, k) + (1 - wk) * V(i + 1, jj, k + 1));
      dv.push_back(wi * wk * (V(i, jj, k) + V(i, jj + 1, k)) / 2 +
                   (1 - wi) * wk * (V(i + 1, jj, k) + V(i + 1, jj + 1, k)) / 2 +
                   wi * (1 - wk) * (V(i, jj, k + 1) + V(i, jj + 1, k + 1)) / 2 +
                   (1 - wi) * (1 - wk) * (V(i + 1, jj, k + 1) + V(i + 1, jj + 1, k + 1)) / 2);
      if (az)
        dw.push_back(wi * (W(i, jj, k) + W(i, jj, k + 1)) / 2 + (1 - wi) * (W(i + 1, jj, k) + W(i + 1, jj, k + 1)) / 2);
      else
        dw.push_back(wi * W(i, jj, k + 1) + (1 - wi) * W(i + 1, jj, k + 1));
      dp.push_back(wi * wk * P(i, jj, k) + (1 - wi) * wk * P(i + 1, jj, k) + wi * (1 - wk) * P(i, jj, k + 1) +
                   (1 - wi) * (1 - wk) * P(i + 1, jj, k + 1));
    }
  } else if (direction == 2 && in(0, ig) && in(1, jg)) {
    const long lo[3] = {i, j, L.s[2]}, hi[3] = {i + 2, j + 2, ek + 1};
    if (int rc = S.load(src, lo, hi)) return rc;
    auto U = [&](long a, long b, long c) { return R(S.f[0].at(a, b, c)); };
    auto V = [&](long a, long b, long c) { return R(S.f[1].at(a, b, c)); };
    auto W = [&](long a, long b, long c) { return R(S.f[2].at(a, b, c)); };
    auto P = [&](long a, long b, long c) { return R(S.f[3].at(a, b, c)); };
    for (long kk = L.s[2]; kk < ek; ++kk) {
      cs.push_back(L.coord(2, kk));
      if (ax)
        du.push_back(wj * (U(i, j, kk) + U(i + 1, j, kk)) / 2 + (1 - wj) * (U(i, j + 1, kk) + U(i + 1, j + 1, kk)) / 2);
      else
        du.push_back(wj * U(i + 1, j, kk) + (1 - wj) * V(i + 1, j + 1, kk));
      if (ay)
        dv.push_back(wi * (V(i, j, kk) + V(i, j + 1, kk)) / 2 + (1 - wi) * (V(i + 1, j, kk) + V(i + 1, j + 1, kk)) / 2);
      else
        dv.push_back(wi * V(i, j + 1, kk) + (1 - wi) * V(i + 1, j + 1, kk));
      dw.push_back(wi * wj * (W(i, j, kk) + W(i, j, kk + 1)) / 2 +
                   (1 - wi) * wj * (W(i + 1, j, kk) + W(i + 1, j, kk + 1)) / 2 +
                   wi * (1 - wj) * (W(i, j + 1, kk) + W(i, j + 1, kk + 1)) / 2 +
                   (1 - wi) * (1 - wj) * (W(i + 1, j + 1, kk) + W(i + 1, j + 1, kk + 1)) / 2);
      dp.push_back(wi * wj * P(i, j, kk) + (1 - wi) * wj * P(i + 1, j, kk) + wi * (1 - wj) * P(i, j + 1, kk) +
                   (1 - wi) * (1 - wj) * P(i + 1, j + 1, kk));
    }
  }
  // stable insertion sort on the coordinate (src/VTKDatExport.cpp:312-338)
  for (size_t a = 1; a < cs.size(); ++a) {
    const R key = cs[a], ku = du[a], kv = dv[a], kw = dw[a], kp = dp[a];
    long b = (long)a - 1;
    while (b >= 0 && cs[b] > key) {
      cs[b + 1] = cs[b];
      du[b + 1] = du[b];
      dv[b + 1] = dv[b];
      dw[b + 1] = dw[b];
      dp[b + 1] = dp[b];
      --b;
    }
    cs[b + 1] = key;
    du[b + 1] = ku;
    dv[b + 1] = kv;
    dw[b + 1] = kw;
    dp[b + 1] = kp;
  }
  FILE *f = std::fopen(filename, "w");
  if (!f) {
    err = std::string("write_dat: cannot open ") + filename;
    return MIFGPU_EINVAL;
  }
  for (size_t a = 0; a < cs.size(); ++a) {
    const double px = direction == 0 ? cs[a] : x, py = direction == 1 ? cs[a] : y, pz = direction == 2 ? cs[a] : z;
    std::fprintf(f, "%.8f %.8f %.8f %.8e %.8e %.8e %.8e\n", px, py, pz, (double)du[a], (double)dv[a], (double)dw[a],
                 (double)dp[a]);
  }
  std::fclose(f);
  return MIFGPU_OK;
}

template <typename R>
int vtk_full(const ExportSource &src, const char *filename, std::string &err) {
  const Layout<R> L(src);
  const long ei = L.s[0] + L.N[0], ej = L.s[1] + L.N[1], ek = L.s[2] + L.N[2];
  State S;
  const long lo[3] = {L.s[0], L.s[1], L.s[2]}, hi[3] = {ei + 1, ej + 1, ek + 1};
  if (int rc = S.load(src, lo, hi)) return rc;
  std::ofstream out(filename);
  if (!out) {
    err = std::string("write_vtk_full_mesh: cannot open ") + filename;
    return MIFGPU_EINVAL;
  }
  // src/VTKDatExport.cpp:596-667, default stream formatting
  out << "# vtk DataFile Version 3.0\n"
      << "pressure mesh solution\n"
      << "ASCII\n"
      << "DATASET STRUCTURED_POINTS\n"
      << "DIMENSIONS " << L.N[0] << ' ' << L.N[1] << ' ' << L.N[2] << '\n'
      << "ORIGIN " << L.mn[0] << " " << L.mn[1] << " " << L.mn[2] << "\n"
      << "SPACING " << L.d[0] << ' ' << L.d[1] << ' ' << L.d[2] << '\n'
      << "POINT_DATA " << L.N[0] * L.N[1] * L.N[2] << '\n';
  auto U = [&](long a, long b, long c) { return R(S.f[0].at(a, b, c)); };
  auto V = [&](long a, long b, long c) { return R(S.f[1].at(a, b, c)); };
  auto W = [&](long a, long b, long c) { return R(S.f[2].at(a, b, c)); };
  auto sweep = [&](const char *name, auto value) {
    out << "SCALARS " << name << " double 1\n"
        << "LOOKUP_TABLE default\n";
    for (long k = L.s[2]; k < ek; ++k)
      for (long j = L.s[1]; j < ej; ++j)
        for (long i = L.s[0]; i < ei; ++i) out << value(i, j, k) << ' ';
  };
  sweep("u", [&](long i, long j, long k) { return (U(i, j, k) + U(i + 1, j, k)) / 2; });
  sweep("v", [&](long i, long j, long k) { return (V(i, j, k) + V(i, j + 1, k)) / 2; });
  sweep("w", [&](long i, long j, long k) { return (W(i, j, k) + W(i, j, k + 1)) / 2; });
  sweep("|u|", [&](long i, long j, long k) {
    const R ux = (U(i, j, k) + U(i + 1, j, k)) / 2;
    const R uy = (V(i, j, k) + V(i, j + 1, k)) / 2;
    const R uz = (W(i, j, k) + W(i, j, k + 1)) / 2;
    return std::sqrt(ux * ux + uy * uy + uz * uz);
  });
  sweep("p", [&](long i, long j, long k) { return R(S.f[3].at(i, j, k)); });
  return out ? MIFGPU_OK : MIFGPU_EINVAL;
}

}  // namespace

int export_vtk(const ExportSource &src, const char *filename, std::string &err) {
  return src.fp64 ? vtk_planes<double>(src, filename, err) : vtk_planes<float>(src, filename, err);
}

int export_dat(const ExportSource &src, const char *filename, int direction, double x, double y, double z,
               std::string &err) {
  return src.fp64 ? dat_line<double>(src, filename, direction, x, y, z, err)
                  : dat_line<float>(src, filename, direction, float(x), float(y), float(z), err);
}

int export_vtk_full_mesh(const ExportSource &src, const char *filename, std::string &err) {
  return src.fp64 ? vtk_full<double>(src, filename, err) : vtk_full<float>(src, filename, err);
}

}  // namespace mifgpu
