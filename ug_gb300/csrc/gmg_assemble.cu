// On-device value assembly for cached topologies: the 3D P1 diffusion
// workload (unit cube, six Kuhn tetrahedra red-refined, the Freudenthal
// triangulation of the cube grid; meshgen.cpp kind 1) assembled straight into
// one instance ("slot") of a batched hierarchy whose topology was built once.
//
// Per level: (1) the coefficient k = exp(g) of every tetrahedron at its
// centroid, g the random-Fourier-feature field of fields.h; (2) per matrix row
// the sum over the (up to 24) tetrahedra at the row's node of k_e h K_p, with
// K_p the stiffness of the unit tetrahedron of type p, written into every
// device copy of the row (FP64 / FP32 block CSR, sliced ELLPACK, inverse
// diagonal); boundary rows become unit Dirichlet rows.  The right-hand side is
// the position-keyed uniform load of fields.h.
//
// Two evaluations of the field.  FP64 (the default of the serving pools):
// the phase of feature m at the centroid (c + delta_p) h of tetrahedron p of
// cell c is phi_m + w_m.c h + w_m.delta_p h, so cos of it is the real part of
// the product of per-axis factors exp(i w_md c_d h) (tabulated per level and
// feature, one sincos per table entry), the factor exp(i phi_m) and the
// tetrahedron's exp(i w_m.delta_p h); a cell then costs two complex
// products per feature and each of its six tetrahedra two FMAs, all in FP64:
// k agrees with the host generator's direct evaluation to ~1e-14 relative
// (both round the phase differently, by |phase| ulp at most).  FP32: the
// phases exactly in 32-bit fixed point (fractions of a turn: for centroid
// lattice coordinates c in units of h/4 the phase is phi + sum_d c_d theta_d
// modulo one turn, theta_d = w_d h / 4 rounded to 2^-32 turn), the sines,
// cosines, angle additions, the sum over features and exp in FP32: ~1e-6
// relative in k, about 50x less FP64-free work.
#include <cmath>
#include <cstdint>
#include <algorithm>
#include <cstring>
#include <mutex>

#include "fields.h"
#include "gmg_internal.h"
#include "gmg_serve.h"

namespace gmg {

namespace {

constexpr int ABLK = 256;
__constant__ double c_kref[6][16];  // stiffness of the unit Kuhn tetrahedra (h = 1, k = 1)
__constant__ int c_perm[6][3];      // the axis order of each tetrahedron's path from (0,0,0) to (1,1,1)

// UG's red refinement (generator kind 3): the six tetrahedra of a lattice
// cell differ from cell to cell and come as masks of the cell's corners (bit
// dx | dy << 1 | dz << 2).  d_ug_shape[mask]: the stiffness of the unit
// tetrahedron on those corners (vertices in ascending corner order, h = 1,
// k = 1), its corners, and the code of its centroid in the cell: 4 delta_d
// in 1..3 per axis, code (4 dx - 1) + 3 (4 dy - 1) + 9 (4 dz - 1).  Masks
// that are no tetrahedron stay zero.
struct UgShape {
  double K[16];
  int corner[4];
  int dcode;
};
__device__ UgShape d_ug_shape[256];
constexpr int UG_DCODES = 27;

// the Kuhn tetrahedra of the unit cube: vertices 0, e_a, e_a + e_b, (1,1,1)
const int kPerms[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};

// P1 stiffness grad(phi_i).grad(phi_j) * vol of one tetrahedron with vertices V
void tet_stiffness(const double V[4][3], double *K) {
  double J[3][3];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) J[r][c] = V[c + 1][r] - V[0][r];
  const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                     J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
  // rows of J^{-1} are the gradients of the barycentric coordinates 1..3
  double Ji[3][3];
  Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
  Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
  Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
  Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det;
  Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
  Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
  Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
  Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
  Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
  double G[4][3];
  for (int d = 0; d < 3; ++d) {
    G[1][d] = Ji[0][d];
    G[2][d] = Ji[1][d];
    G[3][d] = Ji[2][d];
    G[0][d] = -(Ji[0][d] + Ji[1][d] + Ji[2][d]);
  }
  const double vol = std::fabs(det) / 6.0;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) K[i * 4 + j] = vol * (G[i][0] * G[j][0] + G[i][1] * G[j][1] + G[i][2] * G[j][2]);
}

int upload_constants(int device) {
  static std::mutex mu;
  static std::vector<int> done;
  std::lock_guard<std::mutex> lk(mu);
  if ((int)done.size() > device && done[device]) return 0;
  double K[6][16];
  for (int p = 0; p < 6; ++p) {
    double V[4][3] = {{0, 0, 0}};
    for (int a = 1; a < 4; ++a) {
      for (int d = 0; d < 3; ++d) V[a][d] = V[a - 1][d];
      V[a][kPerms[p][a - 1]] += 1.0;
    }
    tet_stiffness(V, K[p]);
  }
  GMG_CUDA(cudaMemcpyToSymbol(c_kref, K, sizeof K));
  GMG_CUDA(cudaMemcpyToSymbol(c_perm, kPerms, sizeof kPerms));
  std::vector<UgShape> sh(256);
  std::memset(sh.data(), 0, sizeof(UgShape) * 256);
  for (int mask = 0; mask < 256; ++mask) {
    if (__builtin_popcount(unsigned(mask)) != 4) continue;
    double V[4][3];
    int a = 0, sum[3] = {0, 0, 0};
    for (int c = 0; c < 8; ++c) {
      if (!((mask >> c) & 1)) continue;
      sh[mask].corner[a] = c;
      for (int d = 0; d < 3; ++d) {
        V[a][d] = double((c >> d) & 1);
        sum[d] += (c >> d) & 1;
      }
      ++a;
    }
    double J[3][3];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) J[r][c] = V[c + 1][r] - V[0][r];
    const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                       J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                       J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    if (det == 0.0) continue;  // four corners of one face
    tet_stiffness(V, sh[mask].K);
    sh[mask].dcode = (sum[0] - 1) + 3 * (sum[1] - 1) + 9 * (sum[2] - 1);
  }
  GMG_CUDA(cudaMemcpyToSymbol(d_ug_shape, sh.data(), sizeof(UgShape) * 256));
  if ((int)done.size() <= device) done.resize(device + 1, 0);
  done[device] = 1;
  return 0;
}

// k of every tetrahedron of a level with Nc cells per axis (element
// ((z Nc + y) Nc + x) 6 + p); prm[m] = (phi, theta_x, theta_y, theta_z) in
// 2^-32 turns, theta per h/4.  One thread per cell: the phase of feature m at
// the centroid of tetrahedron p is the cell's phase (origin, 4 theta per cell
// step) plus a fixed offset delta_{m,p} = (3 e_p0 + 2 e_p1 + e_p2).theta_m,
// so each cell takes one sincos per feature and the six cosines follow by
// angle addition with the offsets' cos / sin tabulated in shared memory.
__global__ void __launch_bounds__(ABLK) cube_field_kernel(int Nc, const uint4 *__restrict__ prm, int M, float amp,
                                                          float *__restrict__ kelem) {
  __shared__ uint4 sp[GMG_FIELD_MAX_M];
  __shared__ float2 sd[GMG_FIELD_MAX_M][6];  // (cos, sin) of delta_{m,p}
  for (int m = threadIdx.x; m < M; m += blockDim.x) {
    const uint4 q = prm[m];
    sp[m] = q;
    const uint32_t th[3] = {q.y, q.z, q.w};
    for (int p = 0; p < 6; ++p) {
      const uint32_t d = 3u * th[c_perm[p][0]] + 2u * th[c_perm[p][1]] + th[c_perm[p][2]];
      float sn, cs;
      sincospif(__uint2float_rn(d) * 4.656612873077392578125e-10f, &sn, &cs);
      sd[m][p] = make_float2(cs, sn);
    }
  }
  __syncthreads();
  const long long nc = (long long)Nc * Nc * Nc;
  for (long long cell = (long long)blockIdx.x * blockDim.x + threadIdx.x; cell < nc;
       cell += (long long)gridDim.x * blockDim.x) {
    const uint32_t cx = uint32_t(cell % Nc) * 4u, cy = uint32_t((cell / Nc) % Nc) * 4u,
                   cz = uint32_t(cell / ((long long)Nc * Nc)) * 4u;
    float g[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int m = 0; m < M; ++m) {
      const uint32_t ph = sp[m].x + cx * sp[m].y + cy * sp[m].z + cz * sp[m].w;
      float s0, c0;
      sincospif(__uint2float_rn(ph) * 4.656612873077392578125e-10f, &s0, &c0);  // angle 2 pi ph / 2^32
#pragma unroll
      for (int p = 0; p < 6; ++p) g[p] += c0 * sd[m][p].x - s0 * sd[m][p].y;  // cos(ph + delta)
    }
#pragma unroll
    for (int p = 0; p < 6; ++p) kelem[cell * 6 + p] = expf(amp * g[p]);
  }
}

// FP64 field, per-axis tables of one level (Nc cells per axis, h = 1 / Nc),
// phases at cell centres: X[m][i] = e^{i w_m0 (i + 1/2) h}, Y[m][j] =
// e^{i w_m1 (j + 1/2) h}, ZP[m][k] = e^{i (phi_m + w_m2 (k + 1/2) h)}.  The
// centroids of the tetrahedra pair up about the cell centre:
// delta_p = 1/2 + eps_q for p = 0, 1, 2 (q = p) and delta = 1/2 - eps_q for
// their partners 5, 3, 4, eps_q = (e_p0 - e_p2) / 4; U[m][q] = (cos, sin) of
// w_m.eps_q h
__global__ void __launch_bounds__(ABLK) cube_field64_tables_kernel(int Nc, double h, int M,
                                                                   const double *__restrict__ w,
                                                                   const double *__restrict__ phi,
                                                                   double2 *__restrict__ X, double2 *__restrict__ Y,
                                                                   double2 *__restrict__ ZP, double2 *__restrict__ U) {
  const int per = 3 * Nc + 3;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= M * per) return;
  const int m = t / per, q = t % per;
  double arg;
  double2 *dst;
  if (q < Nc) {
    arg = w[m * 3] * ((q + 0.5) * h);
    dst = X + (size_t)m * Nc + q;
  } else if (q < 2 * Nc) {
    arg = w[m * 3 + 1] * ((q - Nc + 0.5) * h);
    dst = Y + (size_t)m * Nc + (q - Nc);
  } else if (q < 3 * Nc) {
    arg = phi[m] + w[m * 3 + 2] * ((q - 2 * Nc + 0.5) * h);
    dst = ZP + (size_t)m * Nc + (q - 2 * Nc);
  } else {
    const int p = q - 3 * Nc;  // 0, 1, 2
    arg = h * 0.25 * (w[m * 3 + c_perm[p][0]] - w[m * 3 + c_perm[p][2]]);
    dst = U + (size_t)m * 3 + p;
  }
  double sn, cs;
  sincos(arg, &sn, &cs);
  *dst = make_double2(cs, sn);
}

// FP64 field: k of every tetrahedron of the level (element ((z Nc + y) Nc +
// x) 6 + p).  One block per row (y, z) of cells: the row's factors Y ZP per
// feature and the pair factors U in shared memory; per cell and feature E =
// X YZ = e^{i a0} (a0 the phase at the cell centre), then for each pair
// S += Re E cos u, D += Im E sin u: cos(a0 + u) = S - D, cos(a0 - u) = S + D
__global__ void __launch_bounds__(128) cube_field64_kernel(int Nc, int M, double amp, const double2 *__restrict__ X,
                                                           const double2 *__restrict__ Y,
                                                           const double2 *__restrict__ ZP,
                                                           const double2 *__restrict__ U,
                                                           double *__restrict__ kelem) {
  __shared__ double2 sYZ[GMG_FIELD_MAX_M];
  __shared__ double2 sU[GMG_FIELD_MAX_M * 3];
  const int row = blockIdx.x, j = row % Nc, k = row / Nc;
  for (int m = threadIdx.x; m < M; m += blockDim.x) {
    const double2 b = Y[(size_t)m * Nc + j], c = ZP[(size_t)m * Nc + k];
    sYZ[m] = make_double2(b.x * c.x - b.y * c.y, b.x * c.y + b.y * c.x);
  }
  for (int q = threadIdx.x; q < M * 3; q += blockDim.x) sU[q] = U[q];
  __syncthreads();
  for (int i = threadIdx.x; i < Nc; i += blockDim.x) {
    double S[3] = {0.0, 0.0, 0.0}, D[3] = {0.0, 0.0, 0.0};
    for (int m = 0; m < M; ++m) {
      const double2 a = __ldg(X + (size_t)m * Nc + i), yz = sYZ[m];
      const double er = fma(a.x, yz.x, -a.y * yz.y), ei = fma(a.x, yz.y, a.y * yz.x);
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        S[q] = fma(er, sU[m * 3 + q].x, S[q]);
        D[q] = fma(ei, sU[m * 3 + q].y, D[q]);
      }
    }
    double *ke = kelem + ((size_t)row * Nc + i) * 6;
    // tetrahedra 0, 1, 2 at 1/2 + eps_q; their partners 5, 3, 4 at 1/2 - eps_q
    ke[0] = exp(amp * (S[0] - D[0]));
    ke[5] = exp(amp * (S[0] + D[0]));
    ke[1] = exp(amp * (S[1] - D[1]));
    ke[3] = exp(amp * (S[1] + D[1]));
    ke[2] = exp(amp * (S[2] - D[2]));
    ke[4] = exp(amp * (S[2] + D[2]));
  }
}

__device__ __forceinline__ int lattice_code(int dx, int dy, int dz) { return (dx + 1) + 3 * (dy + 1) + 9 * (dz + 1); }

// UG's mesh, FP32 field: as cube_field_kernel, with the offset of each
// tetrahedron's centroid from its cell's origin looked up by its code (the
// 27 offsets of every feature in shared memory)
__global__ void __launch_bounds__(ABLK) ug_field_kernel(int Nc, const uint4 *__restrict__ prm, int M, float amp,
                                                        const uint8_t *__restrict__ masks,
                                                        float *__restrict__ kelem) {
  extern __shared__ float2 sdu[];  // [M][27]: (cos, sin) of the centroid offsets
  __shared__ uint4 sp[GMG_FIELD_MAX_M];
  for (int q = threadIdx.x; q < M * UG_DCODES; q += blockDim.x) {
    const int m = q / UG_DCODES, c = q % UG_DCODES;
    const uint4 v = prm[m];
    if (c == 0) sp[m] = v;
    const uint32_t d = uint32_t(c % 3 + 1) * v.y + uint32_t((c / 3) % 3 + 1) * v.z + uint32_t(c / 9 + 1) * v.w;
    float sn, cs;
    sincospif(__uint2float_rn(d) * 4.656612873077392578125e-10f, &sn, &cs);
    sdu[q] = make_float2(cs, sn);
  }
  __syncthreads();
  const long long nc = (long long)Nc * Nc * Nc;
  for (long long cell = (long long)blockIdx.x * blockDim.x + threadIdx.x; cell < nc;
       cell += (long long)gridDim.x * blockDim.x) {
    const uint32_t cx = uint32_t(cell % Nc) * 4u, cy = uint32_t((cell / Nc) % Nc) * 4u,
                   cz = uint32_t(cell / ((long long)Nc * Nc)) * 4u;
    int code[6];
#pragma unroll
    for (int t = 0; t < 6; ++t) code[t] = d_ug_shape[masks[cell * 6 + t]].dcode;
    float g[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int m = 0; m < M; ++m) {
      const uint32_t ph = sp[m].x + cx * sp[m].y + cy * sp[m].z + cz * sp[m].w;
      float s0, c0;
      sincospif(__uint2float_rn(ph) * 4.656612873077392578125e-10f, &s0, &c0);
#pragma unroll
      for (int t = 0; t < 6; ++t) {
        const float2 o = sdu[m * UG_DCODES + code[t]];
        g[t] += c0 * o.x - s0 * o.y;
      }
    }
#pragma unroll
    for (int t = 0; t < 6; ++t) kelem[cell * 6 + t] = expf(amp * g[t]);
  }
}

// UG's mesh, FP64 field: V[m][code] = (cos, sin) of w_m.eps h, eps = delta -
// 1/2 the centroid's offset from the cell centre (-1/4, 0 or 1/4 per axis)
__global__ void __launch_bounds__(ABLK) ug_field64_offsets_kernel(double h, int M, const double *__restrict__ w,
                                                                  double2 *__restrict__ V) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= M * UG_DCODES) return;
  const int m = q / UG_DCODES, c = q % UG_DCODES;
  const double ex = 0.25 * double(c % 3 - 1), ey = 0.25 * double((c / 3) % 3 - 1), ez = 0.25 * double(c / 9 - 1);
  const double arg = h * (ex * w[m * 3] + ey * w[m * 3 + 1] + ez * w[m * 3 + 2]);
  double sn, cs;
  sincos(arg, &sn, &cs);
  V[q] = make_double2(cs, sn);
}

// UG's mesh, FP64 field: one block per row (y, z) of cells; per cell and
// feature E = e^{i a0} at the cell centre, then for each tetrahedron
// cos(a0 + u) = Re E cos u - Im E sin u, u its centroid's offset phase
__global__ void __launch_bounds__(128) ug_field64_kernel(int Nc, int M, double amp, const double2 *__restrict__ X,
                                                         const double2 *__restrict__ Y, const double2 *__restrict__ ZP,
                                                         const double2 *__restrict__ V,
                                                         const uint8_t *__restrict__ masks,
                                                         double *__restrict__ kelem) {
  extern __shared__ double2 sV[];  // [M][27]
  __shared__ double2 sYZ[GMG_FIELD_MAX_M];
  const int row = blockIdx.x, j = row % Nc, k = row / Nc;
  for (int m = threadIdx.x; m < M; m += blockDim.x) {
    const double2 b = Y[(size_t)m * Nc + j], c = ZP[(size_t)m * Nc + k];
    sYZ[m] = make_double2(b.x * c.x - b.y * c.y, b.x * c.y + b.y * c.x);
  }
  for (int q = threadIdx.x; q < M * UG_DCODES; q += blockDim.x) sV[q] = V[q];
  __syncthreads();
  for (int i = threadIdx.x; i < Nc; i += blockDim.x) {
    const size_t cell = (size_t)row * Nc + i;
    int code[6];
#pragma unroll
    for (int t = 0; t < 6; ++t) code[t] = d_ug_shape[masks[cell * 6 + t]].dcode;
    double S[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, D[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int m = 0; m < M; ++m) {
      const double2 a = __ldg(X + (size_t)m * Nc + i), yz = sYZ[m];
      const double er = fma(a.x, yz.x, -a.y * yz.y), ei = fma(a.x, yz.y, a.y * yz.x);
#pragma unroll
      for (int t = 0; t < 6; ++t) {
        const double2 v = sV[m * UG_DCODES + code[t]];
        S[t] = fma(er, v.x, S[t]);
        D[t] = fma(ei, v.y, D[t]);
      }
    }
#pragma unroll
    for (int t = 0; t < 6; ++t) kelem[cell * 6 + t] = exp(amp * (S[t] - D[t]));
  }
}

// UG's mesh: one slot's rows of one level, each row summing the tetrahedra
// of its eight cells that contain its node (as cube_assemble_kernel; the
// cells' tetrahedra come from their corner masks)
template <class TK>
__global__ void __launch_bounds__(ABLK) ug_assemble_kernel(
    int nrows, const int *__restrict__ rows, const int *__restrict__ perm, int off, int N,
    const int *__restrict__ rowptr, const int *__restrict__ col, const uint8_t *__restrict__ masks,
    const TK *__restrict__ kelem, double h, double *__restrict__ v64, float *__restrict__ v32,
    const int *__restrict__ c2s, double *__restrict__ sv64, float *__restrict__ sv32, double *__restrict__ dinv64,
    float *__restrict__ dinv32) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nrows) return;
  const int i = rows[q], j = perm[i] - off;
  const int x = j % N, y = (j / N) % N, z = j / (N * N);
  const bool bnd = x == 0 || y == 0 || z == 0 || x == N - 1 || y == N - 1 || z == N - 1;
  double acc[27];
#pragma unroll
  for (int t = 0; t < 27; ++t) acc[t] = 0.0;
  if (!bnd) {
    const int Nc = N - 1;
    for (int cc = 0; cc < 8; ++cc) {  // the cells around the node; the node is their corner cc
      const long long cell = ((long long)(z - ((cc >> 2) & 1)) * Nc + (y - ((cc >> 1) & 1))) * Nc + (x - (cc & 1));
      for (int t = 0; t < 6; ++t) {
        const int mask = masks[cell * 6 + t];
        if (!((mask >> cc) & 1)) continue;
        const UgShape &sh = d_ug_shape[mask];
        const int m = __popc(unsigned(mask) & ((1u << cc) - 1u));
        const double ke = kelem ? double(kelem[cell * 6 + t]) : 1.0;
        for (int b = 0; b < 4; ++b) {
          const int ct = sh.corner[b];
          acc[lattice_code((ct & 1) - (cc & 1), ((ct >> 1) & 1) - ((cc >> 1) & 1), ((ct >> 2) & 1) - ((cc >> 2) & 1))] +=
              ke * sh.K[m * 4 + b];
        }
      }
    }
  }
  for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
    double v;
    if (bnd) {
      v = k == rowptr[i] ? 1.0 : 0.0;
    } else {
      const int jc = perm[col[k]] - off;
      v = h * acc[lattice_code(jc % N - x, (jc / N) % N - y, jc / (N * N) - z)];
    }
    v64[k] = v;
    v32[k] = float(v);
    if (c2s) {
      sv64[c2s[k]] = v;
      sv32[c2s[k]] = float(v);
    }
    if (k == rowptr[i]) {
      dinv64[i] = 1.0 / v;
      dinv32[i] = float(1.0 / v);
    }
  }
}

// the Kuhn tetrahedra as compile-time functions (kPerms above), so that the
// unrolled assembly loops index the row accumulators with constants
__host__ __device__ constexpr int kperm(int p, int k) {
  return p == 0 ? k
       : p == 1 ? (k == 0 ? 0 : k == 1 ? 2 : 1)
       : p == 2 ? (k == 0 ? 1 : k == 1 ? 0 : 2)
       : p == 3 ? (k == 0 ? 1 : k == 1 ? 2 : 0)
       : p == 4 ? (k == 0 ? 2 : k == 1 ? 0 : 1)
                : (k == 0 ? 2 : k == 1 ? 1 : 0);
}
// coordinate d of vertex t of tetrahedron p, relative to its cell's origin
__host__ __device__ constexpr int tvert(int p, int t, int d) {
  return t == 0 ? 0 : t == 3 ? 1 : t == 1 ? int(d == kperm(p, 0)) : int(d == kperm(p, 0) || d == kperm(p, 1));
}
// vertex of tetrahedron p at cell corner cc (bit d = coordinate d), or -1
__host__ __device__ constexpr int tmatch(int p, int cc) {
  return (tvert(p, 0, 0) == (cc & 1) && tvert(p, 0, 1) == ((cc >> 1) & 1) && tvert(p, 0, 2) == ((cc >> 2) & 1)) ? 0
       : (tvert(p, 1, 0) == (cc & 1) && tvert(p, 1, 1) == ((cc >> 1) & 1) && tvert(p, 1, 2) == ((cc >> 2) & 1)) ? 1
       : (tvert(p, 2, 0) == (cc & 1) && tvert(p, 2, 1) == ((cc >> 1) & 1) && tvert(p, 2, 2) == ((cc >> 2) & 1)) ? 2
       : (tvert(p, 3, 0) == (cc & 1) && tvert(p, 3, 1) == ((cc >> 1) & 1) && tvert(p, 3, 2) == ((cc >> 2) & 1)) ? 3
                                                                                                              : -1;
}
// lattice code of vertex t of tetrahedron p seen from the node at corner cc
__host__ __device__ constexpr int tcode(int p, int t, int cc) {
  return (tvert(p, t, 0) - (cc & 1) + 1) + 3 * (tvert(p, t, 1) - ((cc >> 1) & 1) + 1) +
         9 * (tvert(p, t, 2) - ((cc >> 2) & 1) + 1);
}

__device__ __forceinline__ double pick27(const double (&acc)[27], int code) {
  double v = 0.0;
#pragma unroll
  for (int t = 0; t < 27; ++t) v = code == t ? acc[t] : v;
  return v;
}

// one slot's rows of one level (kelem: FP64 or FP32 field)
template <class TK>
__global__ void __launch_bounds__(ABLK) cube_assemble_kernel(
    int nrows, const int *__restrict__ rows, const int *__restrict__ perm, int off, int N,
    const int *__restrict__ rowptr, const int *__restrict__ col, const TK *__restrict__ kelem, double h,
    double *__restrict__ v64, float *__restrict__ v32, const int *__restrict__ c2s, double *__restrict__ sv64,
    float *__restrict__ sv32, double *__restrict__ dinv64, float *__restrict__ dinv32) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nrows) return;
  const int i = rows[q], j = perm[i] - off;
  const int x = j % N, y = (j / N) % N, z = j / (N * N);
  const bool bnd = x == 0 || y == 0 || z == 0 || x == N - 1 || y == N - 1 || z == N - 1;
  double acc[27];
#pragma unroll
  for (int t = 0; t < 27; ++t) acc[t] = 0.0;
  if (!bnd) {
    const int Nc = N - 1;
#pragma unroll
    for (int cc = 0; cc < 8; ++cc) {  // the cells around the node; the node is their corner cc
      const long long cell = ((long long)(z - ((cc >> 2) & 1)) * Nc + (y - ((cc >> 1) & 1))) * Nc + (x - (cc & 1));
#pragma unroll
      for (int p = 0; p < 6; ++p) {
        const int m = tmatch(p, cc);
        if (m < 0) continue;
        const double ke = kelem ? double(kelem[cell * 6 + p]) : 1.0;
#pragma unroll
        for (int t = 0; t < 4; ++t) acc[tcode(p, t, cc)] += ke * c_kref[p][m * 4 + t];
      }
    }
  }
  for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
    double v;
    if (bnd) {
      v = k == rowptr[i] ? 1.0 : 0.0;
    } else {
      const int jc = perm[col[k]] - off;
      v = h * pick27(acc, lattice_code(jc % N - x, (jc / N) % N - y, jc / (N * N) - z));
    }
    v64[k] = v;
    v32[k] = float(v);
    if (c2s) {
      sv64[c2s[k]] = v;
      sv32[c2s[k]] = float(v);
    }
    if (k == rowptr[i]) {
      dinv64[i] = 1.0 / v;
      dinv32[i] = float(1.0 / v);
    }
  }
}

// the position-keyed load on the slot's finest level; x = 0 there
__global__ void __launch_bounds__(ABLK) cube_rhs_kernel(int nrows, const int *__restrict__ rows,
                                                        const int *__restrict__ perm, int off, int N, uint64_t seed,
                                                        double hd, double *__restrict__ b, double *__restrict__ x) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nrows) return;
  const int i = rows[q], j = perm[i] - off;
  const int ix = j % N, iy = (j / N) % N, iz = j / (N * N);
  const bool bnd = ix == 0 || iy == 0 || iz == 0 || ix == N - 1 || iy == N - 1 || iz == N - 1;
  b[i] = bnd ? 0.0 : ugfx::rhs_uniform(seed, ugfx::lattice_key(ix, iy, iz)) * hd;
  x[i] = 0.0;
}

// per-component norms of b over the slot's NEW_DEFECT rows: a fixed grid of
// blocks writes partial sums, the block that draws the last ticket adds them
// in block order (deterministic), writes the norms and resets the ticket
template <int S>
__global__ void __launch_bounds__(ABLK) slot_norm_kernel(int nrows, const int *__restrict__ rows,
                                                         const uint8_t *__restrict__ flags,
                                                         const double *__restrict__ b, double *__restrict__ partial,
                                                         unsigned *__restrict__ ticket, double *__restrict__ out) {
  double acc[S];
#pragma unroll
  for (int r = 0; r < S; ++r) acc[r] = 0.0;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nrows; q += gridDim.x * blockDim.x) {
    const int i = rows[q];
    if (!(flags[i] & F_NEWDEF)) continue;
#pragma unroll
    for (int r = 0; r < S; ++r) acc[r] = fma(b[(size_t)i * S + r], b[(size_t)i * S + r], acc[r]);
  }
  __shared__ double sh[ABLK / 32][S];
  __shared__ bool last;
#pragma unroll
  for (int r = 0; r < S; ++r) {
    double v = acc[r];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5][r] = v;
  }
  __syncthreads();
  if (threadIdx.x < S) {
    double v = 0.0;
    for (int w = 0; w < ABLK / 32; ++w) v += sh[w][threadIdx.x];
    partial[(size_t)blockIdx.x * S + threadIdx.x] = v;
    __threadfence();
  }
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  if (threadIdx.x < S) {
    double v = 0.0;
    for (unsigned k = 0; k < gridDim.x; ++k) v += __ldcg(partial + (size_t)k * S + threadIdx.x);
    out[threadIdx.x] = sqrt(v);
  }
  if (threadIdx.x == 0) *ticket = 0u;
}

unsigned grid_of(long long n) { return unsigned((n + ABLK - 1) / ABLK); }

#define ACHECK(mg)                                                                              \
  do {                                                                                          \
    (mg)->launches++;                                                                           \
    cudaError_t e_ = cudaGetLastError();                                                        \
    if (e_ != cudaSuccess) {                                                                    \
      set_error("%s:%d kernel launch: %s", __FILE__, __LINE__, cudaGetErrorString(e_));         \
      return 1;                                                                                 \
    }                                                                                           \
  } while (0)

}  // namespace

void cube_field_params(uint64_t seed, double corr, double var, int level, std::vector<uint32_t> &prm, float *amp,
                       int *M) {
  ugfx::LogNormalField f(seed, 3, corr, var, GMG_FIELD_MAX_M);
  const double h = 1.0 / double(1 << level), two_pi = 6.283185307179586;
  auto turn = [](double t) -> uint32_t {  // fraction of a turn in [0,1) -> 2^-32 units
    t -= std::floor(t);
    double u = std::floor(t * 4294967296.0 + 0.5);
    return uint32_t(uint64_t(u) & 0xffffffffull);
  };
  prm.resize(size_t(f.M) * 4);
  for (int m = 0; m < f.M; ++m) {
    prm[m * 4] = turn(f.phi[m] / two_pi);
    for (int d = 0; d < 3; ++d) prm[m * 4 + 1 + d] = turn(f.w[size_t(m) * 3 + d] * h / 4.0 / two_pi);
  }
  *amp = float(f.amp);
  *M = f.M;
}

template <class KERN>
static int allow_smem(KERN kern, int bytes) {
  static std::mutex mu;
  static std::vector<std::pair<void *, int>> set;
  std::lock_guard<std::mutex> lk(mu);
  for (auto &e : set)
    if (e.first == (void *)kern && e.second >= bytes) return 0;
  GMG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  set.emplace_back((void *)kern, bytes);
  return 0;
}

int k_cube_field(gmg_mg *mg, int Nc, const uint32_t *prm_dev, int M, float amp, float *kelem,
                 const uint8_t *masks) {
  GMG_CHECK(M <= GMG_FIELD_MAX_M, "field with %d features (at most %d)", M, GMG_FIELD_MAX_M);
  if (upload_constants(mg->device)) return 1;
  const long long nc = (long long)Nc * Nc * Nc;
  const unsigned g = unsigned(std::min<long long>((nc + ABLK - 1) / ABLK, 152LL * 8));
  if (masks) {
    const int smem = M * UG_DCODES * int(sizeof(float2));
    if (allow_smem(ug_field_kernel, smem)) return 1;
    ug_field_kernel<<<g, ABLK, smem, mg->stream>>>(Nc, reinterpret_cast<const uint4 *>(prm_dev), M, amp, masks,
                                                   kelem);
  } else {
    cube_field_kernel<<<g, ABLK, 0, mg->stream>>>(Nc, reinterpret_cast<const uint4 *>(prm_dev), M, amp, kelem);
  }
  ACHECK(mg);
  return 0;
}

int k_cube_field64(gmg_mg *mg, int Nc, const double *w_dev, const double *phi_dev, int M, double amp,
                   double2 *tables, double *kelem, const uint8_t *masks) {
  GMG_CHECK(M <= GMG_FIELD_MAX_M, "field with %d features (at most %d)", M, GMG_FIELD_MAX_M);
  if (upload_constants(mg->device)) return 1;
  double2 *X = tables, *Y = X + (size_t)M * Nc, *ZP = Y + (size_t)M * Nc, *U = ZP + (size_t)M * Nc;
  const int nt = M * (3 * Nc + 3);
  cube_field64_tables_kernel<<<grid_of(nt), ABLK, 0, mg->stream>>>(Nc, 1.0 / double(Nc), M, w_dev, phi_dev, X, Y,
                                                                    ZP, U);
  ACHECK(mg);
  const int bt = std::min(128, std::max(32, (Nc + 31) / 32 * 32));
  if (masks) {
    double2 *V = U + (size_t)M * 3;  // M x 27
    ug_field64_offsets_kernel<<<grid_of(M * UG_DCODES), ABLK, 0, mg->stream>>>(1.0 / double(Nc), M, w_dev, V);
    ACHECK(mg);
    const int smem = M * UG_DCODES * int(sizeof(double2));
    if (allow_smem(ug_field64_kernel, smem)) return 1;
    ug_field64_kernel<<<unsigned(Nc) * unsigned(Nc), bt, smem, mg->stream>>>(Nc, M, amp, X, Y, ZP, V, masks, kelem);
  } else {
    cube_field64_kernel<<<unsigned(Nc) * unsigned(Nc), bt, 0, mg->stream>>>(Nc, M, amp, X, Y, ZP, U, kelem);
  }
  ACHECK(mg);
  return 0;
}

template <class TK>
static int assemble_t(gmg_mg *mg, const Level &L, const SlotLevel &sl, const TK *kelem, double h, const int *c2s) {
  GMG_CHECK(L.s == 1 && L.A.v32 && L.dinv32, "cube assembly: scalar level with FP32 copies expected");
  if (upload_constants(mg->device)) return 1;
  if (sl.masks)
    ug_assemble_kernel<TK><<<grid_of(sl.nrows), ABLK, 0, mg->stream>>>(
        sl.nrows, sl.rows, L.perm_dev, sl.off, sl.N, L.A.rowptr, L.A.col, sl.masks, kelem, h, L.A.v64, L.A.v32,
        c2s, L.sell_v64, L.sell_v32, L.dinv64, L.dinv32);
  else
    cube_assemble_kernel<TK><<<grid_of(sl.nrows), ABLK, 0, mg->stream>>>(
        sl.nrows, sl.rows, L.perm_dev, sl.off, sl.N, L.A.rowptr, L.A.col, kelem, h, L.A.v64, L.A.v32, c2s,
        L.sell_v64, L.sell_v32, L.dinv64, L.dinv32);
  ACHECK(mg);
  return 0;
}

int k_cube_assemble(gmg_mg *mg, const Level &L, const SlotLevel &sl, const float *kelem, double h,
                    const int *c2s) {
  return assemble_t(mg, L, sl, kelem, h, c2s);
}

int k_cube_assemble64(gmg_mg *mg, const Level &L, const SlotLevel &sl, const double *kelem, double h,
                      const int *c2s) {
  return assemble_t(mg, L, sl, kelem, h, c2s);
}

int k_cube_rhs(gmg_mg *mg, const Level &L, const SlotLevel &sl, uint64_t seed, double *b, double *x) {
  const double h = 1.0 / double(sl.N - 1);
  cube_rhs_kernel<<<grid_of(sl.nrows), ABLK, 0, mg->stream>>>(sl.nrows, sl.rows, L.perm_dev, sl.off, sl.N, seed,
                                                               h * h * h, b, x);
  ACHECK(mg);
  return 0;
}

int k_slot_norm(gmg_mg *mg, const Level &L, const SlotLevel &sl, const double *b, double *scratch, double *out) {
  // scratch: SLOT_NORM_BLOCKS * GMG_MAX_S partial sums, then the ticket
  const int nb = int(std::min<long long>(SLOT_NORM_BLOCKS, std::max(1, (sl.nrows + ABLK - 1) / ABLK)));
  unsigned *ticket = reinterpret_cast<unsigned *>(scratch + SLOT_NORM_BLOCKS * GMG_MAX_S);
  switch (L.s) {
    case 1: slot_norm_kernel<1><<<nb, ABLK, 0, mg->stream>>>(sl.nrows, sl.rows, L.flags, b, scratch, ticket, out); break;
    case 2: slot_norm_kernel<2><<<nb, ABLK, 0, mg->stream>>>(sl.nrows, sl.rows, L.flags, b, scratch, ticket, out); break;
    case 3: slot_norm_kernel<3><<<nb, ABLK, 0, mg->stream>>>(sl.nrows, sl.rows, L.flags, b, scratch, ticket, out); break;
    default: set_error("block size %d not compiled", L.s); return 1;
  }
  ACHECK(mg);
  return 0;
}

}  // namespace gmg
