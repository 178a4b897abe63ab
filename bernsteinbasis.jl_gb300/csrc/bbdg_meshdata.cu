// Import of StartUpDG MeshData-shaped arrays (host code, no device work): the packed face
// connectivity from StartUpDG's node-level `mapP` and `Fmask`, and the per-element geometry
// records from the affine metric terms, face-constant scaled normals and Jacobians. With these
// a mesh built by StartUpDG (examples/3d_wave.jl:89-97) runs on the solver unchanged.
#include <cmath>
#include <vector>

#include "bbdg_internal.cuh"

namespace {

// Face node (a, b) of face f in the kernels' ordering (b outer, a inner) -> volume index.
int our_face_vol(int N, int f, int a, int b) { return face_vol(N, f, a, b, 0); }

// Node of the partner face that face node (a, b) meets under orientation o.
int partner_node(int N, int o, int a, int b) {
  const int wgt[3] = {a, b, N - a - b};
  int wn[3];
  for (int v = 0; v < 3; ++v) wn[perm_of(o, v)] = wgt[v];
  return ij2(N, wn[0], wn[1]);
}

}  // namespace

extern "C" int bb_conn_from_mapP(int N, int64_t K, const int32_t* Fmask, const int64_t* mapP,
                                 int32_t* conn_out) {
  if (!valid_degree(N) || K < 1 || K >= (int64_t(1) << 27) || !Fmask || !mapP || !conn_out)
    return BB_ERR_ARG;
  const int Np = np3(N), Nfp = np2(N), NfpT = 4 * Nfp;
  // Fmask position of every volume index, per face (-1: not on that face)
  std::vector<int> pos((size_t)4 * Np, -1);
  for (int f = 0; f < 4; ++f)
    for (int j = 0; j < Nfp; ++j) {
      const int v = Fmask[f * Nfp + j];
      if (v < 0 || v >= Np) return BB_ERR_ARG;
      pos[(size_t)f * Np + v] = j;
    }
  // kernel face-node order <-> Fmask order, per face
  std::vector<int> fm_of_ours((size_t)4 * Nfp), ours_of_fm((size_t)4 * Nfp, -1);
  for (int f = 0; f < 4; ++f) {
    int q = 0;
    for (int b = 0; b <= N; ++b)
      for (int a = 0; a <= N - b; ++a, ++q) {
        const int j = pos[(size_t)f * Np + our_face_vol(N, f, a, b)];
        if (j < 0) return BB_ERR_ARG;  // Fmask does not list this face's nodes
        fm_of_ours[(size_t)f * Nfp + q] = j;
        ours_of_fm[(size_t)f * Nfp + j] = q;
      }
  }
  std::vector<int> part(Nfp);
  for (int64_t e = 0; e < K; ++e)
    for (int f = 0; f < 4; ++f) {
      int64_t e2 = -1;
      int f2 = -1;
      for (int q = 0; q < Nfp; ++q) {
        const int64_t g = mapP[e * NfpT + f * Nfp + fm_of_ours[(size_t)f * Nfp + q]];
        if (g < 0 || g >= K * NfpT) return BB_ERR_ARG;
        const int64_t ge = g / NfpT;
        const int gf = (int)((g % NfpT) / Nfp), gj = (int)(g % Nfp);
        if (q == 0) {
          e2 = ge;
          f2 = gf;
        } else if (ge != e2 || gf != f2) {
          return BB_ERR_ARG;  // one face side must meet one partner face
        }
        part[q] = ours_of_fm[(size_t)gf * Nfp + gj];
      }
      int orient = -1;
      for (int o = 0; o < 6 && orient < 0; ++o) {
        bool ok = true;
        int q = 0;
        for (int b = 0; b <= N && ok; ++b)
          for (int a = 0; a <= N - b; ++a, ++q)
            if (partner_node(N, o, a, b) != part[q]) {
              ok = false;
              break;
            }
        if (ok) orient = o;
      }
      if (orient < 0) return BB_ERR_ARG;  // the node pairing is not a face symmetry
      conn_out[e * 4 + f] = (int32_t)((e2 << 5) | ((int64_t)f2 << 3) | orient);
    }
  return BB_OK;
}

extern "C" int bb_geo_from_meshdata(int64_t K, int dtype, const double* rst9, const double* nJ,
                                    const double* J, void* geo_out) {
  if (K < 1 || !valid_dtype(dtype) || !rst9 || !nJ || !J || !geo_out) return BB_ERR_ARG;
  for (int64_t e = 0; e < K; ++e) {
    double g[BB_GEO_STRIDE] = {0.0};
    for (int m = 0; m < 9; ++m) g[m] = rst9[e * 9 + m];
    if (!(J[e] > 0.0) || !std::isfinite(J[e])) return BB_ERR_ARG;
    g[9] = 1.0 / J[e];
    g[10] = J[e];
    for (int f = 0; f < 4; ++f)
      for (int c = 0; c < 3; ++c) g[12 + 4 * c + f] = nJ[(e * 4 + f) * 3 + c];
    if (dtype == BB_F64) {
      double* o = static_cast<double*>(geo_out) + e * BB_GEO_STRIDE;
      for (int m = 0; m < BB_GEO_STRIDE; ++m) o[m] = g[m];
    } else {
      float* o = static_cast<float*>(geo_out) + e * BB_GEO_STRIDE;
      for (int m = 0; m < BB_GEO_STRIDE; ++m) o[m] = (float)g[m];
    }
  }
  return BB_OK;
}
