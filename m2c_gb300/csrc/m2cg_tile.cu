// Fused MUSCL reconstruction + CheckReconstructedStates + numerical flux of the
// interior faces, with the stage input staged in shared memory by TMA.
//
// Replaces, for primitive-variable reconstruction with constant states at
// material interfaces (the reference's defaults), the face-state passes
// Reconstructor::Reconstruct (Reconstructor.cpp:426-782),
// SpaceOperator::CheckReconstructedStates (SpaceOperator.cpp:2420-2569) and the
// same-material branch of the face loop (SpaceOperator.cpp:1692-1701,
// 1852-1861, 2011-2020): the six face states of a cell never leave the SM.
//
// Layout: a CTA of 128 threads owns a 32 (x) x 4 (y) column of cells and
// marches along z over a chunk of planes.  Each plane of the stage input
// (rho, u, v, w, p; binary64, ghosted) arrives through five 3D tensor-map
// copies of a 36 x 7 box into a five-plane ring in shared memory, one
// mbarrier per ring slot, two planes ahead of the plane being worked on.  A
// thread evaluates the three faces at the minus side of its cell: both face
// states of each (the minus cell's plus state and its own minus state, which
// share one slope difference), the reference's checks on both, then the flux
// when the two cells carry the same material.  Every interior face is
// evaluated once; the faces on the domain boundary, whose outer state the
// boundary condition gives, are evaluated by k_boundary_faces.
//
// FP64 on GB300 runs at two FMAs per clock per SM, so the work here is bound
// by the FP64 pipe, not by HBM: staging the tile in shared memory removes the
// face-state round trip through HBM (6 x 40 B written and read per cell and
// stage) and the scattered per-thread global loads, not FP64 work.
#include "m2cg_internal.h"

namespace m2cg {

namespace tile {
constexpr int TX = 32, TY = 4;           // cells per plane of a tile (one thread each)
constexpr int BX = 36, BY = 7;           // staged box: x from real i0-3, y from real j0-2
constexpr int VSTRIDE = 256;             // doubles per staged array (box 252, padded to 2 KiB)
constexpr int RING = 4;                  // planes k-1 .. k+1 in use, k+2 in flight (k0-2 .. k0+1 at the start)
constexpr int PLANE = 5 * VSTRIDE;       // doubles per ring slot
constexpr uint32_t PLANE_BYTES = 5u * BX * BY * sizeof(double);   // bytes one plane's copies deliver
constexpr long long WAIT_POLLS = 1ll << 22;
}  // namespace tile

// ---- TMA and mbarrier -------------------------------------------------------
__device__ __forceinline__ uint32_t s_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void bar_init(uint64_t* b) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(s_addr(b)) : "memory");
}
__device__ __forceinline__ void bar_expect(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(s_addr(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool bar_wait(uint64_t* b, uint32_t parity, long long max_polls) {
  const uint32_t a = s_addr(b);
  for (long long i = 0; i < max_polls; i++) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}
// One box of a 3D tensor map into shared memory; completion is signalled on
// the mbarrier as transferred bytes.  x must be a multiple of 2 (binary64
// elements, 16-byte rule); y and z may lie outside the tensor (zero fill).
__device__ __forceinline__ void tma_box(void* dst, const CUtensorMap* map, uint64_t* b, int x, int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], "
      "[%2];" ::"r"(s_addr(dst)),
      "l"((unsigned long long)map), "r"(s_addr(b)), "r"(x), "r"(y), "r"(z)
      : "memory");
}

// ---- one face state ---------------------------------------------------------
// Limited slope of one variable from its two one-sided differences (and their
// squares, for van Albada), as in k_reconstruct.
__device__ __forceinline__ double slope(const Params& P, double dq0, double dq1, double a, double b) {
  if (P.limiter == M2CG_LIM_VANALBADA) return van_albada_sq(dq0, dq1, a, b);
  if (P.limiter == M2CG_LIM_GENERALIZED_MINMOD) return gen_minmod(P.minmod_coeff, dq0, dq1);
  return 0.5 * (dq0 + dq1);
}

// Cell access: the staged tile (shared memory) or global memory.
struct SmemCells {
  const double* ring;   // RING slots of PLANE doubles
  const int32_t* id;    // global IDs (ghosted)
  Grid g;
  int i0, j0;
  // a cell: tile x index (i - i0 + 3), tile y index (j - j0 + 2), real k
  struct C { int x, y, k; };
  M2CG_DEV double q(int p, C c) const {
    return ring[((c.k + 2) & (tile::RING - 1)) * tile::PLANE + p * tile::VSTRIDE + c.y * tile::BX + c.x];
  }
  M2CG_DEV int idv(C c) const { return id[g.at(c.x - 3 + i0, c.y - 2 + j0, c.k)]; }
  M2CG_DEV C nb(C c, int d, int s) const {
    if (d == 0) c.x += s;
    else if (d == 1) c.y += s;
    else c.k += s;
    return c;
  }
};
struct GlobalCells {
  const StateSet* S;
  const int32_t* id;
  Grid g;
  typedef int64_t C;
  M2CG_DEV double q(int p, C c) const { return S->q[p][c]; }
  M2CG_DEV int idv(C c) const { return id[c]; }
  M2CG_DEV C nb(C c, int d, int s) const { return c + (d == 0 ? (int64_t)s : d == 1 ? s * g.sy : s * g.sz); }
};

// Face f (vl, vr, vb, vt, vk, vf) of cell c before any check
// (Reconstructor.cpp:426-716), with the arithmetic of k_reconstruct.
template <class A>
M2CG_DEV void raw_face(const Params& P, const A& a, typename A::C c, int f, int myid, double* out) {
  double q[5];
#pragma unroll
  for (int p = 0; p < 5; p++) q[p] = a.q(p, c);
  if (P.rec_type == M2CG_REC_CONSTANT) {
#pragma unroll
    for (int p = 0; p < 5; p++) out[p] = q[p];
    return;
  }
  const int d = f >> 1;
  typename A::C cm = a.nb(c, d, -1), cp = a.nb(c, d, 1);
  const bool zero = P.slope_zero && (a.idv(cm) != myid || a.idv(cp) != myid);
  const double h = (f & 1) ? 0.5 : -0.5;
#pragma unroll
  for (int p = 0; p < 5; p++) {
    double dq0 = q[p] - a.q(p, cm);
    double dq1 = a.q(p, cp) - q[p];
    double s = slope(P, dq0, dq1, __dmul_rn(dq0, dq0), __dmul_rn(dq1, dq1));
    if (zero) s = 0.0;
    out[p] = fma(h, s, q[p]);
  }
}

// The checks a face state goes through, given its unchecked value V (updated
// in place): the reference's revert of the first nonphysical face state of the
// cell to the cell value (Reconstructor.cpp:722-778; the earlier faces of the
// cell are evaluated only when this one is nonphysical), then
// CheckReconstructedStates (SpaceOperator.cpp:2446-2484): a state that clipping
// would change reverts to the cell value.  Counts clipped and nonphysical
// states as k_reconstruct does.
template <class A>
M2CG_DEV void check_face(const Params& P, const A& a, typename A::C c, int f, int myid, double* V, int& nclip,
                         int& nbad) {
  const DevMat& M = P.mats.m[myid];
  if (P.rec_type != M2CG_REC_CONSTANT && eos_bad5_fast(M, V)) {
    bool first = true;
    for (int e = 0; e < f && first; e++) {
      double W[5];
      raw_face(P, a, c, e, myid, W);
      first = !eos_bad5_fast(M, W);
    }
    if (first)
#pragma unroll
      for (int p = 0; p < 5; p++) V[p] = a.q(p, c);
  }
  double t[5] = {V[0], V[1], V[2], V[3], V[4]};
  if (eos_clip_fast(M, t)) {
#pragma unroll
    for (int p = 0; p < 5; p++) V[p] = a.q(p, c);
    nclip++;
  }
  nbad += eos_bad5_fast(M, V);
}

__device__ __forceinline__ bool tile_flux(const Params& P, int dir, const double* Vm, const double* Vp, int id,
                                          double* F) {
  const DevMat& M = P.mats.m[id];
  if (P.flux == M2CG_FLUX_HLLC) return flux_hllc_fast(M, dir, Vm, Vp, F);
  if (P.flux == M2CG_FLUX_LLF) return flux_llf2(M, M, dir, Vm, Vp, F);
  return flux_genroe(M, dir, Vm, Vp, P.roe_delta, F);
}

__device__ __forceinline__ void warp_count(unsigned long long* c, int v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd(c, (unsigned long long)v);
}

// ---------------------------------------------------------------------------
// Face states of one cell in direction d (Reconstructor.cpp:426-716): one
// limited slope per variable gives the minus (vl / vb / vk) and plus (vr / vt /
// vf) states; then the cell's revert chain (the first nonphysical state in the
// order vl, vr, vb, vt, vk, vf reverts to the cell value; `done` carries the
// chain across directions, Reconstructor.cpp:722-778) and
// CheckReconstructedStates (SpaceOperator.cpp:2446-2484), counted as
// k_reconstruct + store_faces count them.  The same arithmetic as k_reconstruct.
__device__ __forceinline__ void cell_faces_dir(const Params& P, const DevMat& M, const SmemCells& a, SmemCells::C c,
                                               int d, const double* q, int myid, double* vm, double* vp,
                                               bool& done, int& nclip, int& nbad) {
  if (P.rec_type == M2CG_REC_CONSTANT) {
#pragma unroll
    for (int p = 0; p < 5; p++) { vm[p] = q[p]; vp[p] = q[p]; }
  } else {
    const SmemCells::C cm = a.nb(c, d, -1), cp = a.nb(c, d, 1);
    const bool zero = P.slope_zero && (a.idv(cm) != myid || a.idv(cp) != myid);
#pragma unroll
    for (int p = 0; p < 5; p++) {
      const double dq0 = q[p] - a.q(p, cm);
      const double dq1 = a.q(p, cp) - q[p];
      double sl = slope(P, dq0, dq1, __dmul_rn(dq0, dq0), __dmul_rn(dq1, dq1));
      if (zero) sl = 0.0;
      vm[p] = fma(-0.5, sl, q[p]);
      vp[p] = fma(0.5, sl, q[p]);
    }
    if (!done && eos_bad5_fast(M, vm)) {
#pragma unroll
      for (int p = 0; p < 5; p++) vm[p] = q[p];
      done = true;
    }
    if (!done && eos_bad5_fast(M, vp)) {
#pragma unroll
      for (int p = 0; p < 5; p++) vp[p] = q[p];
      done = true;
    }
  }
  double t[5] = {vm[0], vm[1], vm[2], vm[3], vm[4]};
  if (eos_clip_fast(M, t)) {
#pragma unroll
    for (int p = 0; p < 5; p++) vm[p] = q[p];
    nclip++;
  }
  nbad += eos_bad5_fast(M, vm);
#pragma unroll
  for (int p = 0; p < 5; p++) t[p] = vp[p];
  if (eos_clip_fast(M, t)) {
#pragma unroll
    for (int p = 0; p < 5; p++) vp[p] = q[p];
    nclip++;
  }
  nbad += eos_bad5_fast(M, vp);
}

// One checked face state of a cell outside the tile's own cells (a halo cell,
// or the cell below the chunk): raw state plus the checks of check_face, not
// counted (its own tile counts it).
__device__ __forceinline__ void halo_face(const Params& P, const SmemCells& a, SmemCells::C c, int f, double* V) {
  const int hid = a.idv(c);
  raw_face(P, a, c, f, hid, V);
  int dc = 0, db = 0;
  check_face(P, a, c, f, hid, V, dc, db);
}

// ---------------------------------------------------------------------------
// Interior faces of the z-chunk [k0, k1) of one 32 x 4 column.  F[d*5+p][c]:
// flux of the face at the minus side of cell c in direction d (same-material
// faces only; interface faces come from the Riemann pass).
//
// Per plane: two warps first evaluate the states the tile's first column and
// row need from the cells just outside it; then, direction by direction, every
// thread reconstructs its own cell (one limited slope per variable, the
// k_reconstruct arithmetic), hands the plus state to the neighbour that needs
// it -- vr by a warp shuffle (x runs along the warp), vt through shared memory
// (y runs across the warps), vf in registers until the next plane -- and
// evaluates the flux of its minus face in that direction.  Holding one
// direction's states at a time keeps the register count down.
__global__ void __launch_bounds__(128, 4) k_recon_flux_tile(const __grid_constant__ TileMaps maps, Params P,
                                                        const int32_t* __restrict__ id, double* const* F,
                                                        unsigned long long* cnt, int zchunk) {
  extern __shared__ __align__(128) double ring_raw[];
  __shared__ __align__(8) uint64_t bars[tile::RING];
  __shared__ double s_vt[tile::TY][5][tile::TX];      // vt of the tile's rows (read by the next row)
  __shared__ double s_vt_halo[5][tile::TX];           // vt of row j0-1
  __shared__ double s_vr_halo[5][tile::TY];           // vr of column i0-1
  // TMA destinations on 128-byte boundaries (the launch adds 128 bytes of slack)
  double* ring = ring_raw + ((128u - (s_addr(ring_raw) & 127u)) & 127u) / sizeof(double);
  const Grid& g = P.g;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int i0 = blockIdx.x * tile::TX, j0 = blockIdx.y * tile::TY;
  const int k0 = blockIdx.z * zchunk, k1 = min(g.nz, k0 + zchunk);
  const int i = i0 + tx, j = j0 + ty;
  const bool active = i < g.nx && j < g.ny;
  // plane kk (real index, k0-2 .. k1) of the ring: slot (kk + 2) % RING; its
  // n-th load into that slot completes phase n
  static_assert((tile::RING & (tile::RING - 1)) == 0, "ring slots: a power of two");
  auto slot = [](int kk) { return (kk + 2) & (tile::RING - 1); };
  auto issue = [&](int kk) {
    double* dst = ring + slot(kk) * tile::PLANE;
    uint64_t* b = &bars[slot(kk)];
    bar_expect(b, tile::PLANE_BYTES);
#pragma unroll
    for (int p = 0; p < 5; p++) tma_box(dst + p * tile::VSTRIDE, &maps.v[p], b, i0 - 2, j0 - 1, kk + 1);
  };
  auto parity = [&](int kk) { return (uint32_t)(((kk - (k0 - 2)) / tile::RING) & 1); };
  if (threadIdx.x == 0) {
    for (int s = 0; s < tile::RING; s++) bar_init(&bars[s]);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0)
    for (int kk = k0 - 2; kk <= min(k0 + 1, k1); kk++) issue(kk);
  const SmemCells a{ring, id, g, i0, j0};
  const int64_t sy = g.sy, sz = g.sz;
  int nclip = 0, nbad = 0;
  double vf_prev[5];   // checked vf of the cell below (the minus state of the z face)
  bool ok = true;
  for (int k = k0; k < k1; k++) {
    __syncthreads();   // every thread is done with plane k-2's slot and with s_vt
    if (threadIdx.x == 0 && k > k0 && k + 2 <= k1) issue(k + 2);
    bool w = true;
    if (k == k0)
      for (int kk = k0 - 2; kk < k0 && w; kk++) w = bar_wait(&bars[slot(kk)], parity(kk), tile::WAIT_POLLS);
    w = w && bar_wait(&bars[slot(k)], parity(k), tile::WAIT_POLLS);
    w = w && bar_wait(&bars[slot(k + 1)], parity(k + 1), tile::WAIT_POLLS);
    ok = __syncthreads_and(w);   // one decision for the whole CTA
    if (!ok) break;
    const SmemCells::C cc{tx + 3, ty + 2, k};
    if (k == k0) {
      // the first plane of the chunk: vf of the cell below, the one use of plane
      // k0-2, whose slot then takes plane k0+2
      if (k > 0 && active) halo_face(P, a, a.nb(cc, 2, -1), 5, vf_prev);
      __syncthreads();
      if (threadIdx.x == 0 && k + 2 <= k1) issue(k + 2);
    }
    // states from the cells just outside the tile: vt of row j0-1 (warp 3),
    // vr of column i0-1 (warp 2, one lane per row)
    if (ty == 3 && j0 > 0 && i < g.nx) {
      double V[5];
      halo_face(P, a, SmemCells::C{tx + 3, 1, k}, 3, V);
#pragma unroll
      for (int p = 0; p < 5; p++) s_vt_halo[p][tx] = V[p];
    }
    if (ty == 2 && tx < tile::TY && i0 > 0 && j0 + tx < g.ny) {
      double V[5];
      halo_face(P, a, SmemCells::C{2, tx + 2, k}, 1, V);
#pragma unroll
      for (int p = 0; p < 5; p++) s_vr_halo[p][tx] = V[p];
    }
    int myid = 0;
    double q[5] = {0, 0, 0, 0, 0};
    if (active) {
      myid = id[g.at(i, j, k)];
#pragma unroll
      for (int p = 0; p < 5; p++) q[p] = a.q(p, cc);
    }
    const DevMat& M = P.mats.m[myid];
    const int64_t c = g.at(i, j, k);
    bool done = false;   // the cell's revert chain, carried across directions
    int bad = 0;
    // x: own vl, vr; vr of the left neighbour by shuffle (lane 0: the halo)
    {
      double vl[5], vr[5] = {0, 0, 0, 0, 0};
      if (active) cell_faces_dir(P, M, a, cc, 0, q, myid, vl, vr, done, nclip, nbad);
      double vrl[5];
#pragma unroll
      for (int p = 0; p < 5; p++) vrl[p] = __shfl_up_sync(0xffffffffu, vr[p], 1);
      __syncthreads();   // the halo states are written
      if (active && i > 0) {
        if (tx == 0)
#pragma unroll
          for (int p = 0; p < 5; p++) vrl[p] = s_vr_halo[p][ty];
        if (id[c - 1] == myid) {
          double Fl[5];
          bad += !tile_flux(P, 0, vrl, vl, myid, Fl);
#pragma unroll
          for (int p = 0; p < 5; p++) F[p][c] = Fl[p];
        }
      }
    }
    // y: own vb, vt; vt of the row below from shared memory (row 0: the halo)
    {
      double vb[5], vt[5];
      if (active) {
        cell_faces_dir(P, M, a, cc, 1, q, myid, vb, vt, done, nclip, nbad);
#pragma unroll
        for (int p = 0; p < 5; p++) s_vt[ty][p][tx] = vt[p];
      }
      __syncthreads();   // every row's vt is written
      if (active && j > 0) {
        double vtm[5];
#pragma unroll
        for (int p = 0; p < 5; p++) vtm[p] = ty > 0 ? s_vt[ty - 1][p][tx] : s_vt_halo[p][tx];
        if (id[c - sy] == myid) {
          double Fl[5];
          bad += !tile_flux(P, 1, vtm, vb, myid, Fl);
#pragma unroll
          for (int p = 0; p < 5; p++) F[5 + p][c] = Fl[p];
        }
      }
    }
    // z: own vk, vf; vf of the cell below kept from the previous plane
    if (active) {
      double vk[5], vf[5];
      cell_faces_dir(P, M, a, cc, 2, q, myid, vk, vf, done, nclip, nbad);
      if (k > 0 && id[c - sz] == myid) {
        double Fl[5];
        bad += !tile_flux(P, 2, vf_prev, vk, myid, Fl);
#pragma unroll
        for (int p = 0; p < 5; p++) F[10 + p][c] = Fl[p];
      }
#pragma unroll
      for (int p = 0; p < 5; p++) vf_prev[p] = vf[p];
    }
    nbad += bad;
  }
  if (!ok) {
    // a copy did not complete in time: flag it, give the copies in flight a
    // bounded chance to land, and leave the tile's fluxes unwritten
    if (threadIdx.x == 0) {
      atomicAdd(&cnt[CNT_TILE_TIMEOUT], 1ull);
      for (int s = 0; s < tile::RING; s++) bar_wait(&bars[s], 0, tile::WAIT_POLLS >> 4);
    }
    __syncthreads();
    return;
  }
  warp_count(&cnt[CNT_CLIPFACE], nclip);
  warp_count(&cnt[CNT_BAD], nbad);
}

// ---------------------------------------------------------------------------
// The faces on the domain boundary (one thread each, six sides): the real
// cell's face state on the boundary side with its checks (counted by the
// tile kernel, which evaluates all six states of every cell), the ghost's face
// state by boundary condition (Reconstructor.cpp:807-889) with the boundary
// branch of CheckReconstructedStates (SpaceOperator.cpp:2486-2535), then the
// flux, stored at the face's plus cell like every other face (the ghost on
// the upper sides).
__global__ void k_boundary_faces(Params P, StateSet S, const int32_t* __restrict__ id, double* const* F,
                                 unsigned long long* cnt) {
  int side, i, j, k, ii, jj, kk;
  if (!ghost_face_cell(P.g, (int64_t)blockIdx.x * blockDim.x + threadIdx.x, side, i, j, k, ii, jj, kk)) return;
  const Grid& g = P.g;
  const int64_t gc = g.at(i, j, k), r = g.at(ii, jj, kk);
  const int d = side >> 1;
  const bool upper = side & 1;
  GlobalCells a{&S, id, g};
  const int rid = id[r], gid = id[gc];
  int nclip = 0, nbad = 0;
  // the real cell's state on this side: vl/vb/vk (lower) or vr/vt/vf (upper),
  // counted where the tile kernel evaluates the cell's six states
  const int f = 2 * d + (upper ? 1 : 0);
  double Vr[5];
  raw_face(P, a, r, f, rid, Vr);
  {
    int dc = 0, db = 0;
    check_face(P, a, r, f, rid, Vr, dc, db);
  }
  // the ghost's state facing the domain
  double t[5];
  const int bc = P.bc[side];
  if (bc == M2CG_BC_INLET || bc == M2CG_BC_INLET2) {
#pragma unroll
    for (int p = 0; p < 5; p++) t[p] = S.q[p][gc];
  } else {
#pragma unroll
    for (int p = 0; p < 5; p++) t[p] = Vr[p];
    if (bc == M2CG_BC_SYMMETRY || bc == M2CG_BC_SLIPWALL) t[1 + d] *= -1.0;
    else if (bc == M2CG_BC_STICKWALL) { t[1] *= -1.0; t[2] *= -1.0; t[3] *= -1.0; }
  }
  {
    const DevMat& M = P.mats.m[gid];
    double u[5] = {t[0], t[1], t[2], t[3], t[4]};
    if (eos_clip(M, u)) {
#pragma unroll
      for (int p = 0; p < 5; p++) t[p] = S.q[p][gc];
      nclip++;
    }
    nbad += eos_bad5(M, t);
  }
  // flux of the face, stored at its plus cell
  const int64_t pc = upper ? gc : r;
  const int pid = upper ? gid : rid, mid = upper ? rid : gid;
  if (mid == pid) {
    double Fl[5];
    nbad += !tile_flux(P, d, upper ? Vr : t, upper ? t : Vr, pid, Fl);
#pragma unroll
    for (int p = 0; p < 5; p++) F[d * 5 + p][pc] = Fl[p];
  }
  if (nclip) atomicAdd(&cnt[CNT_CLIPFACE], (unsigned long long)nclip);
  if (nbad) atomicAdd(&cnt[CNT_BAD], (unsigned long long)nbad);
}

// ---- host side --------------------------------------------------------------
static size_t tile_smem_bytes() { return (size_t)tile::RING * tile::PLANE * sizeof(double) + 128; }

// The tile path covers primitive-variable reconstruction (or none) with
// constant states at material interfaces on a grid whose rows are a multiple
// of 16 bytes (nx even).
bool tile_supported(const Params& P) {
  if (P.rec_type != M2CG_REC_CONSTANT && P.rec_var != M2CG_VAR_PRIMITIVE) return false;
  if (P.mp_recon != M2CG_MPREC_CONSTANT) return false;
  return (P.g.px % 2) == 0;
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// Tensor maps of the five primitive arrays of a state set.  Returns false when
// the driver entry point or an encode is unavailable (the caller keeps the
// three-kernel path).
bool tile_maps(const Params& P, const StateSet& S, TileMaps* out) {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !f) {
      cudaGetLastError();
      return false;
    }
    fn = (EncodeTiledFn)f;
  }
  const cuuint64_t dims[3] = {(cuuint64_t)P.g.px, (cuuint64_t)P.g.py, (cuuint64_t)P.g.pz};
  const cuuint64_t strides[2] = {(cuuint64_t)P.g.px * sizeof(double), (cuuint64_t)P.g.px * P.g.py * sizeof(double)};
  const cuuint32_t box[3] = {tile::BX, tile::BY, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  for (int p = 0; p < 5; p++) {
    if (fn(&out->v[p], CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, (void*)S.q[p], dims, strides, box, estr,
           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return false;
  }
  return true;
}

cudaError_t tile_prepare() {
  return cudaFuncSetAttribute(k_recon_flux_tile, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tile_smem_bytes());
}

// Interior faces (tile kernel) and boundary faces of one stage input.
void launch_recon_flux_tile(cudaStream_t s, const TileMaps& maps, const Params& P, const StateSet& S,
                            const int32_t* id, double* const* F, unsigned long long* cnt, int zchunk) {
  dim3 grid((P.g.nx + tile::TX - 1) / tile::TX, (P.g.ny + tile::TY - 1) / tile::TY, (P.g.nz + zchunk - 1) / zchunk);
  k_recon_flux_tile<<<grid, 128, tile_smem_bytes(), s>>>(maps, P, id, F, cnt, zchunk);
  int64_t ng = 2 * ((int64_t)P.g.ny * P.g.nz + (int64_t)P.g.nx * P.g.nz + (int64_t)P.g.nx * P.g.ny);
  k_boundary_faces<<<(int)((ng + 127) / 128), 128, 0, s>>>(P, S, id, F, cnt);
}

}  // namespace m2cg
