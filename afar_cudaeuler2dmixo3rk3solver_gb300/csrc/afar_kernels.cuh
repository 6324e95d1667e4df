// AFAR stage kernels for sm_103a: reconstruct, BVD switch, adaptive flux, fused residual gather +
// SSP-RK3 update + boundary ghosts, plus the setup kernels that build the device operators.
//
// Device layout (one mesh):
//   per cell      W[Nc+Nb] (ghosts after the cells), U/U0[Nc], grad[2Nc], lim[Nc], si[Nc+Nb]
//   per slot      slot-major "[slot][ldc]" arrays, slot i of every cell contiguous so that a warp
//                 of consecutive cells reads one coalesced row per slot:
//                   sten[maxS]            global stencil cell ids
//                   cf[maxM]              signed face ids (+f+1 owner side, -(f+1) neighbour side)
//                   lsm[maxM]             least-squares gradient rows (M1, M2)
//                   sg[maxM], sr[maxM]    face offset from the cell centre; (delta r, fraction)
//                   wts[maxM*(maxS+1)]    O3 weights of the cell's side of each face
//   per face      on[Nf], fd[Nf] (face offsets from owner and neighbour), fs[Nf+Nb] (Sf, |Sf|),
//                 dtg[Nf] (CFL geometry), fv[2Nf] face values, flux[Nf+Nb]
// Every kernel here is one thread per cell or per face; every output element has one writer, so
// the stage is deterministic (no atomics except the min of the time step, which is exact).
#pragma once

#include "afar_policy.cuh"

namespace afar {

struct StepCtl {
  unsigned long long dt_bits;  // running min of the CFL time step (bits of a non-negative double)
  double t;                    // simulated time
  double t_end;                // > 0: clip the last step to land on t_end
  double dt_fixed;             // > 0: fixed step, else CFL step
  double cfl;
  double last_dt;
  long long steps;
  unsigned err;  // bit 0: a bounded device wait gave up (the stage's results are not valid)
  double write_interval;  // > 0: land on its multiples like OpenFOAM's adjustableRunTime
  long long write_index;  // write times passed
};

// The step of the current RK step: fixed or CFL, spread over the steps left to the next write time
// when write times are set, clipped to t_end; <= 0 means "no step".  The write-time rule is
// OpenFOAM's Time::adjustDeltaT for writeControl adjustableRunTime (the reference application
// sets each step with runTime.setDeltaT, cudaEuler2DmixO3RK3solver.cpp:44-48): with r the time to
// the next write, n = floor(r/dt - small) + 1 steps of r/n, the change held within [dt/5, 2 dt].
__device__ __forceinline__ double step_dt(const StepCtl* c) {
  double dt = c->dt_fixed > 0.0 ? c->dt_fixed : __longlong_as_double((long long)c->dt_bits);
  if (c->write_interval > 0.0) {
    const double r = (double)(c->write_index + 1) * c->write_interval - c->t;
    if (r > 0.0) {
      const double nd = r / (floor(r / dt - 1e-15) + 1.0);
      dt = nd >= dt ? fmin(nd, 2.0 * dt) : fmax(nd, 0.2 * dt);
    }
  }
  if (c->t_end > 0.0) dt = fmin(dt, c->t_end - c->t);
  return dt;
}

// The SSP-RK3 coefficients of one stage: U = b1 Un + b2 U + b3 dt R (truncated decimals, reference
// GPUevolve.cu:222-225), their float-pair splits for the mixed policy (computed on the host so no
// thread converts them), and the first/last-stage flags.
struct StageCoef {
  double b1, b2, b3;
  float b1h, b1l, b2h, b2l;
  int first, last;
};

template <class P>
struct StageArgs {
  using S = typename P::S;
  using G = typename P::G;
  int Nc, Nf, Nb, ldc, maxS, maxM;
  // operators (read-only)
  const V2<double>* cellC;    // Nc+Nb cell centres, ghosts = boundary face centres
  const int2* on;             // Nf (owner, neighbour)
  const V4<G>* fd;            // Nf (xf-x_own, yf-y_own, xf-x_nei, yf-y_nei)
  const V4<G>* fs;            // Nf+Nb (Sfx, Sfy, magSf, 0)
  const V2<double>* dtg;      // Nf (delta r, fraction) of the CFL estimate
  const V2<double>* bn;       // Nb unit normal of each boundary face
  const uint8_t* btype;       // Nb cudaEulerBCs label
  const double* vol;          // Nc
  const double* vinv;         // Nc 1/V (policies without the reference's divisions)
  const float* vinvf;         // Nc 1/V as float (mixed)
  const uint8_t* nS;          // Nc stencil size
  const uint8_t* nM;          // Nc faces per cell (compact stencil size)
  const uint8_t* tileS;       // ceil(Nc/128): the largest stencil size of each 128-cell tile
  const int* sten;            // [maxS][ldc]
  const int* cf;              // [maxM][ldc]
  const V2<S>* lsm;           // [maxM][ldc]
  const V2<G>* sg;            // [maxM][ldc]
  const V2<S>* sr;            // [maxM][ldc]
  const S* wts;               // [maxM*(maxS+1)][ldc]
  const struct TileMaps* tmaps;  // mixed: TMA tensor maps of the operator rows (tile-staged reconstruct)
  // state and stage intermediates
  V4<typename P::W>* W;       // Nc+Nb
  V4<double>* U;              // Nc conserved state (mixed: DF4 float pairs, same 32 bytes)
  V4<double>* U0;             // Nc state at the start of the step (mixed: DF4)
  V4<G>* grad;                // 2Nc
  V4<S>* lim;                 // Nc
  int8_t* si;                 // 2(Nc+Nb): [2c] troubled-cell flag, [2c+1] final switch type
  V4<G>* fv;                  // 2Nf
  V4<typename P::F>* flux;    // Nf+Nb
  StepCtl* ctl;
  V4<double>* res_dbg;        // optional residual dump (parity hook)
  double R, Cv, invR, gamma;
  float gm1f, invRf;  // gamma - 1 and 1/R as floats (mixed)
  float Rf, Cvf, gRf;  // R, Cv and gamma*R as floats (mixed)
  double px, py;       // periods of a periodic mesh (0: none); setup kernels only
  const V2<float>* dtgf;  // Nf (delta r, fraction) as floats (mixed Courant estimate)
  // the optional multi-point face flux (ng > 0 points per face; 0: the face-centre flux)
  int ng;
  const S* wg;       // [(maxM*ng)*(maxS+1)][ldc] O3 weights at the face Gauss points, per cell slot
  const V2<G>* sgk;  // [maxM*ng][ldc] point minus cell centre, per cell slot
  const V2<G>* fgk;  // [Nf*ng] point minus face centre
  V4<G>* fvg;        // [2Nf*ng] face values at the points ((2f + side)*ng + k)
  G gw[4];           // the points' weights, normalised to sum to one
};

// limiterProcess (reference cudaLimiter.h:35-50)
template <class S, class G>
__device__ __forceinline__ void limiter_process(S& limiter, S& phif, const S phic, const S phiMax, const S phiMin,
                                                const G gx, const G gy, const G dx, const G dy) {
  phif = phic;
  phif += gx * dx + gy * dy;
  const S d2 = phif - phic;
  const S d1 = (phif < phic) * (phiMin - phic) + (phif >= phic) * (phiMax - phic);
  S yy = fmn(S(2), S(0.5) * d1 / (d2 + (d2 >= S(0)) * AFAR_LIT(S, 1e-10) - (d2 < S(0)) * AFAR_LIT(S, 1e-10)));
  const bool valid = (fab(d2) >= AFAR_LIT(S, 1e-5));
  yy = valid * yy + (1 - valid) * S(1);
  limiter = fmn(limiter, yy);
}

// limiterProcess for the mixed policy: the same ratio with selects and the fast float division
// (2 ulp, MUFU reciprocal); the ratio feeds a min() with 2 and 1, so a rounding apart is all it
// changes.
__device__ __forceinline__ void limiter_process_fast(float& limiter, float& phif, const float phic, const float phiMax,
                                                     const float phiMin, const float gx, const float gy,
                                                     const float dx, const float dy) {
  phif = phic;
  phif += gx * dx + gy * dy;
  const float d2 = phif - phic;
  const float d1 = phif < phic ? phiMin - phic : phiMax - phic;
  const float yy = fabsf(d2) >= 1e-5f ? fminf(2.f, __fdividef(0.5f * d1, d2 + (d2 >= 0.f ? 1e-10f : -1e-10f))) : 1.f;
  limiter = fminf(limiter, yy);
}

// Faces per cell: triangles and quadrilaterals, the only cells the reference's quadrature accepts
// (d2GaussQuadrature.C:65-148); the stencil upload rejects larger compact stencils.
constexpr int kMaxFaces = 4;

// reconstruct, register-pass variant for the mixed policy (the autotuner's alternative to the
// tile-staged kernel): LS gradient, stencil min/max, raw limiter, O3 RBF face values of this
// cell's side of each internal face, troubled-cell flag.
// One pass over the stencil: each member's state is gathered once and feeds the gradient and
// min/max (compact members) and the O3 sums of every face side at once, all in registers.  The
// loads of a batch of members (indices, gathers, weights) are issued together, so several are in
// flight per thread; no shared memory, so occupancy is set by registers alone.  Every sum is
// still accumulated in stencil order, as in the reference.
template <class P>
__device__ __forceinline__ void recon_reg_body(const StageArgs<P>& a, const int blk) {
  using S = typename P::S;
  using G = typename P::G;
  using WT = typename P::W;
  const int c = blk * blockDim.x + threadIdx.x;
  if (c >= a.Nc) return;
  const int ldc = a.ldc;
  const int nS = a.nS[c], nM = a.nM[c];
  const int wrow = a.maxS + 1;
  int fid[kMaxFaces];
  bool inner[kMaxFaces];
  V2<S> lm[kMaxFaces];
#pragma unroll
  for (int fi = 0; fi < kMaxFaces; ++fi) {
    fid[fi] = fi < nM ? a.cf[fi * ldc + c] : 1;
    inner[fi] = fi < nM && abs(fid[fi]) - 1 < a.Nf;
    lm[fi] = fi < nM ? a.lsm[fi * ldc + c] : V2<S>{S(0), S(0)};
  }
  const V4<WT> wc = a.W[c];
  const S pc = (S)wc.x, uxc = (S)wc.y, uyc = (S)wc.z, tc = (S)wc.w;
  // O3 sums in difference form: sum_i w_i phi_i = phi_c + sum_{i>0} w_i (phi_i - phi_c), since the
  // weights of every face side sum to one.  In FP32 this drops the error phi_c * (sum of the float
  // weights' rounding), which is the same every step and grows like a change of scheme; what
  // remains is rounding relative to the neighbour differences.
  G acc[kMaxFaces][4];
#pragma unroll
  for (int fi = 0; fi < kMaxFaces; ++fi) acc[fi][0] = acc[fi][1] = acc[fi][2] = acc[fi][3] = G(0);
  G gPx = 0, gPy = 0, gUxx = 0, gUxy = 0, gUyx = 0, gUyy = 0, gTx = 0, gTy = 0;
  S pMax = pc, pMin = pc, uxMax = uxc, uxMin = uxc, uyMax = uyc, uyMin = uyc, tMax = tc, tMin = tc;
  S pn[kMaxFaces];  // pressure of the cell across each face
  {  // members 0..3: the face neighbours (compact stencil) come first
    int j[kMaxFaces];
#pragma unroll
    for (int u = 0; u < kMaxFaces; ++u) j[u] = u < nS ? a.sten[u * ldc + c] : c;
    V4<WT> wj[kMaxFaces];
#pragma unroll
    for (int u = 0; u < kMaxFaces; ++u) wj[u] = a.W[j[u]];
    S wv[kMaxFaces][kMaxFaces];
#pragma unroll
    for (int u = 0; u < kMaxFaces; ++u)
#pragma unroll
      for (int fi = 0; fi < kMaxFaces; ++fi)
        wv[u][fi] = (u < nS && inner[fi]) ? a.wts[(size_t)(fi * wrow + u + 1) * ldc + c] : S(0);
#pragma unroll
    for (int u = 0; u < kMaxFaces; ++u) {
      if (u < nS) {
        const S vx = (S)wj[u].x, vy = (S)wj[u].y, vz = (S)wj[u].z, vw = (S)wj[u].w;
        const S dp = vx - pc, dux = vy - uxc, duy = vz - uyc, dt = vw - tc;
        if (u < nM) {  // reference :148-169 and :190-205
          const S M1 = lm[u].x, M2 = lm[u].y;
          gPx += M1 * dp;
          gPy += M2 * dp;
          gUxx += M1 * dux;
          gUyx += M2 * dux;
          gUxy += M1 * duy;
          gUyy += M2 * duy;
          gTx += M1 * dt;
          gTy += M2 * dt;
          pMax = fmx(vx, pMax);
          pMin = fmn(vx, pMin);
          uxMax = fmx(vy, uxMax);
          uxMin = fmn(vy, uxMin);
          uyMax = fmx(vz, uyMax);
          uyMin = fmn(vz, uyMin);
          tMax = fmx(vw, tMax);
          tMin = fmn(vw, tMin);
          pn[u] = vx;
        }
#pragma unroll
        for (int fi = 0; fi < kMaxFaces; ++fi) {
          acc[fi][0] += wv[u][fi] * dp;
          acc[fi][1] += wv[u][fi] * dux;
          acc[fi][2] += wv[u][fi] * duy;
          acc[fi][3] += wv[u][fi] * dt;
        }
      }
    }
  }
  constexpr int U = sizeof(WT) == 4 ? 4 : 2;
  for (int ci0 = kMaxFaces; ci0 < nS; ci0 += U) {  // the rest of the stencil: O3 sums only
    int j[U];
#pragma unroll
    for (int u = 0; u < U; ++u) j[u] = (ci0 + u < nS) ? a.sten[(ci0 + u) * ldc + c] : c;
    V4<WT> wj[U];
#pragma unroll
    for (int u = 0; u < U; ++u) wj[u] = a.W[j[u]];
    S wv[U][kMaxFaces];
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int fi = 0; fi < kMaxFaces; ++fi)
        wv[u][fi] = (ci0 + u < nS && inner[fi]) ? a.wts[(size_t)(fi * wrow + ci0 + u + 1) * ldc + c] : S(0);
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (ci0 + u < nS) {
        const S dp = (S)wj[u].x - pc, dux = (S)wj[u].y - uxc, duy = (S)wj[u].z - uyc, dt = (S)wj[u].w - tc;
#pragma unroll
        for (int fi = 0; fi < kMaxFaces; ++fi) {
          acc[fi][0] += wv[u][fi] * dp;
          acc[fi][1] += wv[u][fi] * dux;
          acc[fi][2] += wv[u][fi] * duy;
          acc[fi][3] += wv[u][fi] * dt;
        }
      }
    }
  }
  a.grad[2 * c] = V4<G>{gPx, gPy, gUxx, gUxy};
  a.grad[2 * c + 1] = V4<G>{gUyx, gUyy, gTx, gTy};

  const S SMALL = AFAR_LIT(S, 1e-5), VSMALL = AFAR_LIT(S, 1e-10);
  V4<S> L;
  int8_t flag0;
  if (fab(tMax - tMin) < VSMALL) {  // reference :208-233
    L = V4<S>{S(1), S(1), S(1), S(1)};
#pragma unroll
    for (int fi = 0; fi < kMaxFaces; ++fi) {
      if (!inner[fi]) continue;
      const bool isNei = fid[fi] < 0;
      const int f = abs(fid[fi]) - 1;
      const V2<G> d = a.sg[fi * ldc + c];
      const G dx = d.x, dy = d.y;
      V4<G> o;
      o.x = (G)(pc) + gPx * dx + gPy * dy;
      o.y = (G)(uxc) + gUxx * dx + gUyx * dy;
      o.z = (G)(uyc) + gUxy * dx + gUyy * dy;
      o.w = (G)(tc) + gTx * dx + gTy * dy;
      a.fv[2 * f + isNei] = o;
    }
    flag0 = 0;
  } else {  // reference :235-314
    S lp = S(2), lux = S(2), luy = S(2), lt = S(2);
    S smooth = S(0);
    bool notTrouble = true;
#pragma unroll
    for (int fi = 0; fi < kMaxFaces; ++fi) {
      if (!inner[fi]) continue;
      const bool isNei = fid[fi] < 0;
      const int f = abs(fid[fi]) - 1;
      const V2<G> d = a.sg[fi * ldc + c];
      const G dx = d.x, dy = d.y;
      const V2<S> rf = a.sr[fi * ldc + c];
      const S deltaR = rf.x, fraction = rf.y;
      const G pf = (G)pc + acc[fi][0], uxf = (G)uxc + acc[fi][1], uyf = (G)uyc + acc[fi][2], tf = (G)tc + acc[fi][3];
      S phif;
      V4<G> o;
      limiter_process_fast(lp, phif, pc, pMax, pMin, gPx, gPy, dx, dy);
      o.x = pick<P>(fab(pMax - pMin) >= SMALL, fab(pMax - pMin) < SMALL, pf, phif);
      notTrouble = phif > S(0);
      smooth = fmx(smooth, __fdividef(fab((S(1) - fraction) * pc + fraction * pn[fi] - phif), deltaR) +
                               (pf <= S(0)) * AFAR_LIT(S, 1e20) + (phif <= S(0)) * AFAR_LIT(S, 1e20));
      limiter_process_fast(lux, phif, uxc, uxMax, uxMin, gUxx, gUyx, dx, dy);
      o.y = pick<P>(fab(uxMax - uxMin) >= SMALL, fab(uxMax - uxMin) < SMALL, uxf, phif);
      limiter_process_fast(luy, phif, uyc, uyMax, uyMin, gUxy, gUyy, dx, dy);
      o.z = pick<P>(fab(uyMax - uyMin) >= SMALL, fab(uyMax - uyMin) < SMALL, uyf, phif);
      limiter_process_fast(lt, phif, tc, tMax, tMin, gTx, gTy, dx, dy);
      o.w = pick<P>(fab(tMax - tMin) >= SMALL, fab(tMax - tMin) < SMALL, tf, phif);
      notTrouble = phif > S(0);
      a.fv[2 * f + isNei] = o;
    }
    L.x = fmx(lp, S(0)) * notTrouble;
    L.y = fmx(lux, S(0)) * notTrouble;
    L.z = fmx(luy, S(0)) * notTrouble;
    L.w = fmx(lt, S(0)) * notTrouble;
    smooth = __fdividef(smooth, S(0.5) * (pMax + pMin) * notTrouble + VSMALL);
    flag0 = (smooth > S(1));
  }
  a.lim[c] = L;
  a.si[2 * c] = flag0;
}

// ---------------------------------------------------------------- mixed reconstruct, tile-staged
// One CTA per 128-cell tile.  The tile's slice of every per-cell operator row (face ids, LS rows,
// face offsets, (dr, fraction), stencil ids, O3 weights) and the cells' own states are contiguous
// 128-element runs of the slot-major arrays, so the CTA fetches them with the TMA unit (one tiled
// load per array from its tensor map, one bulk copy of the states, two mbarriers) instead of
// per-thread loads: ~50 KB per tile in flight from seven lanes, while registers stay free for the
// stencil gathers, which hit L2.  One load per array rather than one per row: the fetch was bound
// by the number of copies issued, not by their bytes.
constexpr int kTile = 128;
// Test hooks of the tile's bounded waits (afar_debug_wait_injection): the wait limit in SM clocks,
// and bytes added to the transaction count the first barrier of every tile expects (never issued,
// so that barrier cannot complete and its wait runs out).  2^31 clocks and no extra bytes in normal
// operation.
static __device__ long long g_tile_wait_limit = 1ll << 31;
static __device__ unsigned g_tile_extra_tx = 0;
// Tensor maps of the mixed policy's slot-major operator rows, one tiled TMA load per array and
// tile: face ids [maxM][ldc] and the LS / face-geometry rows (float pairs, as 2 ldc floats), boxes
// of 128 cells x maxM rows; stencil ids, a box of 128 cells x S rows for each stencil size S; O3
// weights [maxM][maxS+1][ldc], a box of 128 cells x rows 1..S x maxM slots for each S (row 0, the
// cell's own weight, drops out of the difference-form sums).  A tile loads the boxes of its own
// largest stencil, so no row past it is fetched.
struct TileMaps {
  CUtensorMap cf, lsm, sg, sr;
  CUtensorMap sten[AFAR_MAX_VALID_STENCIL_SIZE];
  CUtensorMap wts[AFAR_MAX_VALID_STENCIL_SIZE];
};
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n" ::
          "r"(smem_addr(dst)),
      "l"(map), "r"(x), "r"(y), "r"(smem_addr(bar))
      : "memory");
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z,
                                            unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];\n" ::"r"(smem_addr(dst)),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
      : "memory");
}

struct ReconTile {
  unsigned off_cf, off_lsm, off_sg, off_sr, off_sten, off_wts, off_w, off_bar, bytes;
};
__host__ __device__ inline ReconTile recon_tile_layout(const int maxM, const int maxS) {
  ReconTile L;
  unsigned o = 0;
  L.off_cf = o;
  o += maxM * kTile * 4;
  L.off_lsm = o;
  o += maxM * kTile * 8;
  L.off_sg = o;
  o += maxM * kTile * 8;
  L.off_sr = o;
  o += maxM * kTile * 8;
  L.off_sten = o;
  o += maxS * kTile * 4;
  L.off_wts = o;
  o += maxM * (maxS + 1) * kTile * 4;
  L.off_w = o;
  o += kTile * 16;
  L.off_bar = o;  // two mbarriers: the gather inputs, then the rest
  L.bytes = o + 16;
  return L;
}

// Issues the loads of tile `blk` (lanes 0-6 of warp 0): six tiled TMA loads of its operator rows
// (TileMaps) and one bulk copy of its own states.  The x coordinate of every box is the tile's
// first cell (a multiple of 128 elements: 512 or 1024 bytes, so 16-byte aligned); boxes reaching
// past the row ends of the last tile read zeros and count their full size.  Two barriers: bar[0]
// covers what the stencil gathers need (face ids, stencil ids, own states), bar[1] the LS rows,
// face geometry and O3 weights, so the first gathers are in flight while the weights still stream
// in.  Smem rows hold 128 cells: face ids [maxM][128], stencil ids [S][128], LS and geometry
// [maxM][128] pairs, weights [maxM][S][128] (S = the tile's largest stencil).
template <class P>
__device__ __forceinline__ void recon_tile_fetch(const StageArgs<P>& a, const int blk, const ReconTile& L,
                                                 unsigned char* sm, unsigned long long* bar) {
  const int lane = threadIdx.x;
  const int c0 = blk * kTile;
  const int M = a.maxM, S = a.tileS[blk];
  const TileMaps* tm = a.tmaps;
  if (lane == 0) {
    const unsigned nw = (unsigned)min(kTile, a.Nc - c0);  // cells of the tile
    mbar_arrive_expect_tx(bar, kTile * 4 * (M + S) + nw * 16 + g_tile_extra_tx);
    mbar_arrive_expect_tx(bar + 1, kTile * 8 * 3 * M + kTile * 4 * S * M);
  }
  __syncwarp();
  switch (lane) {
    case 0: tma_load_2d(sm + L.off_cf, &tm->cf, c0, 0, bar); break;
    case 1: tma_load_2d(sm + L.off_sten, &tm->sten[S - 1], c0, 0, bar); break;
    case 2: bulk_to_smem(sm + L.off_w, a.W + c0, (unsigned)min(kTile, a.Nc - c0) * 16u, bar); break;
    case 3: tma_load_2d(sm + L.off_lsm, &tm->lsm, 2 * c0, 0, bar + 1); break;
    case 4: tma_load_2d(sm + L.off_sg, &tm->sg, 2 * c0, 0, bar + 1); break;
    case 5: tma_load_2d(sm + L.off_sr, &tm->sr, 2 * c0, 0, bar + 1); break;
    case 6: tma_load_3d(sm + L.off_wts, &tm->wts[S - 1], c0, 1, 0, bar + 1); break;
    default: break;
  }
}

// reconstruct (reference cudaLimiter.h:53-316) for the mixed policy from the staged tile: LS
// gradient, stencil min/max, raw limiter, O3 RBF face values of this cell's side of each internal
// face, troubled-cell flag.  One pass over the stencil: each member's state is gathered once (in
// batches of 8, all in flight) and feeds the gradient and min/max (compact members) and the O3 sums
// of every face side; every sum is accumulated in stencil order, as in the reference.  NF: the
// largest number of faces of a cell (3 on all-triangle meshes, else 4).
template <class P, int NF>
__device__ __forceinline__ void recon_tile_body(const StageArgs<P>& a, const int blk, unsigned char* sm) {
  using S = typename P::S;
  using G = typename P::G;
  using WT = typename P::W;
  const ReconTile L = recon_tile_layout(a.maxM, a.maxS);
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(sm + L.off_bar);
  const int t = threadIdx.x;
  if (t == 0) {
    mbar_init(bar, 1);
    mbar_init(bar + 1, 1);
  }
  __syncthreads();
  if (t < 32) recon_tile_fetch(a, blk, L, sm, bar);
  const int c = blk * kTile + t;
  const int nS = c < a.Nc ? a.nS[c] : 0, nM = c < a.Nc ? a.nM[c] : 0;
  const long long limit = g_tile_wait_limit;
  // leaving: every copy into this block's shared memory must have landed first
  auto give_up = [&]() {
    if (t == 0) atomicOr(&a.ctl->err, 1u);
    mbar_wait_bounded(bar, 0, limit);
    mbar_wait_bounded(bar + 1, 0, limit);
  };
  if (!mbar_wait_bounded(bar, 0, limit)) return give_up();
  if (c >= a.Nc) {
    if (!mbar_wait_bounded(bar + 1, 0, limit)) give_up();
    return;
  }
  const int* s_cf = reinterpret_cast<const int*>(sm + L.off_cf);
  const V2<S>* s_lsm = reinterpret_cast<const V2<S>*>(sm + L.off_lsm);
  const V2<G>* s_sg = reinterpret_cast<const V2<G>*>(sm + L.off_sg);
  const V2<S>* s_sr = reinterpret_cast<const V2<S>*>(sm + L.off_sr);
  const int* s_sten = reinterpret_cast<const int*>(sm + L.off_sten);
  const S* s_wts = reinterpret_cast<const S*>(sm + L.off_wts);
  const V4<WT>* s_w = reinterpret_cast<const V4<WT>*>(sm + L.off_w);
  const int wrow = a.tileS[blk];  // weight rows of a face slot in shared memory (members 1..S)

  int fid[NF];
  bool inner[NF];
#pragma unroll
  for (int fi = 0; fi < NF; ++fi) {
    fid[fi] = fi < nM ? s_cf[fi * kTile + t] : 1;
    inner[fi] = fi < nM && abs(fid[fi]) - 1 < a.Nf;
  }
  const V4<WT> wc = s_w[t];
  const S pc = (S)wc.x, uxc = (S)wc.y, uyc = (S)wc.z, tc = (S)wc.w;
  constexpr int U = 8;
  V4<WT> wj[U];  // the first batch of stencil states, gathered before the weights have landed
#pragma unroll
  for (int u = 0; u < U; ++u)
    if (u < nS) wj[u] = a.W[s_sten[u * kTile + t]];
  if (!mbar_wait_bounded(bar + 1, 0, limit)) return give_up();
  // O3 weights of boundary-face and missing slots are zero in the operator rows (setup), so only
  // slots past this mesh's largest cell (a batch may stage fewer rows than NF) are skipped
  const int nfm = a.maxM;
  G acc[NF][4];  // O3 sums in difference form, as in recon_reg_body
#pragma unroll
  for (int fi = 0; fi < NF; ++fi) acc[fi][0] = acc[fi][1] = acc[fi][2] = acc[fi][3] = G(0);
  G gPx = 0, gPy = 0, gUxx = 0, gUxy = 0, gUyx = 0, gUyy = 0, gTx = 0, gTy = 0;
  S pMax = pc, pMin = pc, uxMax = uxc, uxMin = uxc, uyMax = uyc, uyMin = uyc, tMax = tc, tMin = tc;
  S pn[NF];  // pressure of the cell across each face
#pragma unroll
  for (int fi = 0; fi < NF; ++fi) pn[fi] = S(0);
  for (int ci0 = 0; ci0 < nS; ci0 += U) {
    if (ci0 > 0) {
#pragma unroll
      for (int u = 0; u < U; ++u)
        if (ci0 + u < nS) wj[u] = a.W[s_sten[(ci0 + u) * kTile + t]];
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int ci = ci0 + u;
      if (ci < nS) {
        const S vx = (S)wj[u].x, vy = (S)wj[u].y, vz = (S)wj[u].z, vw = (S)wj[u].w;
        const S dp = vx - pc, dux = vy - uxc, duy = vz - uyc, dt = vw - tc;
        if (ci < nM) {  // the face neighbours (compact stencil) come first: reference :148-169, :190-205
          const V2<S> lm = s_lsm[ci * kTile + t];
          const S M1 = lm.x, M2 = lm.y;
          gPx += M1 * dp;
          gPy += M2 * dp;
          gUxx += M1 * dux;
          gUyx += M2 * dux;
          gUxy += M1 * duy;
          gUyy += M2 * duy;
          gTx += M1 * dt;
          gTy += M2 * dt;
          pMax = fmx(vx, pMax);
          pMin = fmn(vx, pMin);
          uxMax = fmx(vy, uxMax);
          uxMin = fmn(vy, uxMin);
          uyMax = fmx(vz, uyMax);
          uyMin = fmn(vz, uyMin);
          tMax = fmx(vw, tMax);
          tMin = fmn(vw, tMin);
#pragma unroll
          for (int fi = 0; fi < NF; ++fi)
            if (fi == ci) pn[fi] = vx;
        }
#pragma unroll
        for (int fi = 0; fi < NF; ++fi) {
          const S wv = fi < nfm ? s_wts[(fi * wrow + ci) * kTile + t] : S(0);
          acc[fi][0] += wv * dp;
          acc[fi][1] += wv * dux;
          acc[fi][2] += wv * duy;
          acc[fi][3] += wv * dt;
        }
      }
    }
  }
  a.grad[2 * c] = V4<G>{gPx, gPy, gUxx, gUxy};
  a.grad[2 * c + 1] = V4<G>{gUyx, gUyy, gTx, gTy};

  const S SMALL = AFAR_LIT(S, 1e-5), VSMALL = AFAR_LIT(S, 1e-10);
  V4<S> Lm;
  int8_t flag0;
  if (fab(tMax - tMin) < VSMALL) {  // reference :208-233
    Lm = V4<S>{S(1), S(1), S(1), S(1)};
#pragma unroll
    for (int fi = 0; fi < NF; ++fi) {
      if (!inner[fi]) continue;
      const bool isNei = fid[fi] < 0;
      const int f = abs(fid[fi]) - 1;
      const V2<G> d = s_sg[fi * kTile + t];
      const G dx = d.x, dy = d.y;
      V4<G> o;
      o.x = (G)(pc) + gPx * dx + gPy * dy;
      o.y = (G)(uxc) + gUxx * dx + gUyx * dy;
      o.z = (G)(uyc) + gUxy * dx + gUyy * dy;
      o.w = (G)(tc) + gTx * dx + gTy * dy;
      a.fv[2 * f + isNei] = o;
    }
    flag0 = 0;
  } else {  // reference :235-314
    S lp = S(2), lux = S(2), luy = S(2), lt = S(2);
    S smooth = S(0);
    bool notTrouble = true;
#pragma unroll
    for (int fi = 0; fi < NF; ++fi) {
      if (!inner[fi]) continue;
      const bool isNei = fid[fi] < 0;
      const int f = abs(fid[fi]) - 1;
      const V2<G> d = s_sg[fi * kTile + t];
      const G dx = d.x, dy = d.y;
      const V2<S> rf = s_sr[fi * kTile + t];
      const S deltaR = rf.x, fraction = rf.y;
      const G pf = (G)pc + acc[fi][0], uxf = (G)uxc + acc[fi][1], uyf = (G)uyc + acc[fi][2], tf = (G)tc + acc[fi][3];
      S phif;
      V4<G> o;
      limiter_process_fast(lp, phif, pc, pMax, pMin, gPx, gPy, dx, dy);
      o.x = pick<P>(fab(pMax - pMin) >= SMALL, fab(pMax - pMin) < SMALL, pf, phif);
      notTrouble = phif > S(0);
      smooth = fmx(smooth, __fdividef(fab((S(1) - fraction) * pc + fraction * pn[fi] - phif), deltaR) +
                               (pf <= S(0)) * AFAR_LIT(S, 1e20) + (phif <= S(0)) * AFAR_LIT(S, 1e20));
      limiter_process_fast(lux, phif, uxc, uxMax, uxMin, gUxx, gUyx, dx, dy);
      o.y = pick<P>(fab(uxMax - uxMin) >= SMALL, fab(uxMax - uxMin) < SMALL, uxf, phif);
      limiter_process_fast(luy, phif, uyc, uyMax, uyMin, gUxy, gUyy, dx, dy);
      o.z = pick<P>(fab(uyMax - uyMin) >= SMALL, fab(uyMax - uyMin) < SMALL, uyf, phif);
      limiter_process_fast(lt, phif, tc, tMax, tMin, gTx, gTy, dx, dy);
      o.w = pick<P>(fab(tMax - tMin) >= SMALL, fab(tMax - tMin) < SMALL, tf, phif);
      notTrouble = phif > S(0);
      a.fv[2 * f + isNei] = o;
    }
    Lm.x = fmx(lp, S(0)) * notTrouble;
    Lm.y = fmx(lux, S(0)) * notTrouble;
    Lm.z = fmx(luy, S(0)) * notTrouble;
    Lm.w = fmx(lt, S(0)) * notTrouble;
    smooth = __fdividef(smooth, S(0.5) * (pMax + pMin) * notTrouble + VSMALL);
    flag0 = (smooth > S(1));
  }
  a.lim[c] = Lm;
  a.si[2 * c] = flag0;
}

// reconstruct for the FP64-heavy policies (ref, fp64): the stencil values are staged in shared
// memory in batches (indices, then gathers), then each face side's O3 sum runs over the staged
// values with its weights loaded eight at a time.  These policies are bound by the FP64 pipe, so
// the kernel keeps the per-face loop (no work on missing face slots) and a small register set.
template <class P>
__device__ __forceinline__ void recon_staged_body(const StageArgs<P>& a, const int blk) {
  using S = typename P::S;
  using G = typename P::G;
  using WT = typename P::W;
  // fp64 stages only the compact stencil (kCompact), ref the whole stencil
  constexpr bool kCompact = P::id == PolicyFP64::id;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V4<S>* sv = reinterpret_cast<V4<S>*>(smem_raw);  // [maxM or maxS][blockDim] staged stencil values
  const int t = threadIdx.x, B = blockDim.x;
  const int c = blk * B + t;
  if (c >= a.Nc) return;
  const int ldc = a.ldc;
  const int nS = a.nS[c], nM = a.nM[c];
  const V4<WT> wc = a.W[c];
  const S pc = (S)wc.x, uxc = (S)wc.y, uyc = (S)wc.z, tc = (S)wc.w;
  // fp64: only the compact stencil (the face neighbours, at most kMaxFaces) is staged: the
  // gradient, the min/max and the uniform-cell test need nothing else, and only cells that are not
  // uniform read the rest of the stencil, in their O3 loop.  32-byte values make whole-stencil
  // staging the occupancy limit (3 blocks an SM); with it, 4.  The ref policy's 16-byte values
  // leave room for the whole stencil, which its smooth-flow cells reuse across faces.
  if constexpr (!kCompact) {
    constexpr int GB = 4;
    for (int i0 = 0; i0 < nS; i0 += GB) {
      int j[GB];
#pragma unroll
      for (int u = 0; u < GB; ++u) j[u] = (i0 + u < nS) ? a.sten[(i0 + u) * ldc + c] : c;
      V4<WT> wj[GB];
#pragma unroll
      for (int u = 0; u < GB; ++u) wj[u] = a.W[j[u]];
#pragma unroll
      for (int u = 0; u < GB; ++u)
        if (i0 + u < nS) sv[(i0 + u) * B + t] = V4<S>{(S)wj[u].x, (S)wj[u].y, (S)wj[u].z, (S)wj[u].w};
    }
  } else {
    int j[kMaxFaces];
#pragma unroll
    for (int u = 0; u < kMaxFaces; ++u) j[u] = u < nM ? a.sten[u * ldc + c] : c;
    V4<WT> wj[kMaxFaces];
#pragma unroll
    for (int u = 0; u < kMaxFaces; ++u) wj[u] = a.W[j[u]];
#pragma unroll
    for (int u = 0; u < kMaxFaces; ++u)
      if (u < nM) sv[u * B + t] = V4<S>{(S)wj[u].x, (S)wj[u].y, (S)wj[u].z, (S)wj[u].w};
  }

  G gPx = 0, gPy = 0, gUxx = 0, gUxy = 0, gUyx = 0, gUyy = 0, gTx = 0, gTy = 0;
  for (int i = 0; i < nM; ++i) {  // reference :148-169
    const V2<S> m = a.lsm[i * ldc + c];
    const S M1 = m.x, M2 = m.y;
    const V4<S> v = sv[i * B + t];
    S dphi = v.x - pc;
    gPx += M1 * dphi;
    gPy += M2 * dphi;
    dphi = v.y - uxc;
    gUxx += M1 * dphi;
    gUyx += M2 * dphi;
    dphi = v.z - uyc;
    gUxy += M1 * dphi;
    gUyy += M2 * dphi;
    dphi = v.w - tc;
    gTx += M1 * dphi;
    gTy += M2 * dphi;
  }
  a.grad[2 * c] = V4<G>{gPx, gPy, gUxx, gUxy};
  a.grad[2 * c + 1] = V4<G>{gUyx, gUyy, gTx, gTy};

  S pMax = pc, pMin = pc, uxMax = uxc, uxMin = uxc, uyMax = uyc, uyMin = uyc, tMax = tc, tMin = tc;
  for (int i = 0; i < nM; ++i) {  // reference :190-205
    const V4<S> v = sv[i * B + t];
    pMax = fmx(v.x, pMax);
    pMin = fmn(v.x, pMin);
    uxMax = fmx(v.y, uxMax);
    uxMin = fmn(v.y, uxMin);
    uyMax = fmx(v.z, uyMax);
    uyMin = fmn(v.z, uyMin);
    tMax = fmx(v.w, tMax);
    tMin = fmn(v.w, tMin);
  }

  const S SMALL = AFAR_LIT(S, 1e-5), VSMALL = AFAR_LIT(S, 1e-10);
  V4<S> L;
  int8_t flag0;
  if (fab(tMax - tMin) < VSMALL) {  // reference :208-233
    L = V4<S>{S(1), S(1), S(1), S(1)};
    for (int fi = 0; fi < nM; ++fi) {
      int f = a.cf[fi * ldc + c];
      const bool isNei = (f < 0);
      f = abs(f) - 1;
      if (f >= a.Nf) continue;
      const V2<G> d = a.sg[fi * ldc + c];
      const G dx = d.x, dy = d.y;
      V4<G> o;
      o.x = (G)(pc) + gPx * dx + gPy * dy;
      o.y = (G)(uxc) + gUxx * dx + gUyx * dy;
      o.z = (G)(uyc) + gUxy * dx + gUyy * dy;
      o.w = (G)(tc) + gTx * dx + gTy * dy;
      a.fv[2 * f + isNei] = o;
    }
    flag0 = 0;
  } else {  // reference :235-314
    S lp = S(2), lux = S(2), luy = S(2), lt = S(2);
    S smooth = S(0);
    bool notTrouble = true;
    for (int fi = 0; fi < nM; ++fi) {
      int f = a.cf[fi * ldc + c];
      const bool isNei = (f < 0);
      f = abs(f) - 1;
      if (f >= a.Nf) continue;
      const V2<G> d = a.sg[fi * ldc + c];
      const G dx = d.x, dy = d.y;
      const V2<S> rf = a.sr[fi * ldc + c];
      const S deltaR = rf.x, fraction = rf.y;
      const S* w = a.wts + (size_t)(fi * (a.maxS + 1)) * ldc + c;
      S wk = w[0];
      G pf = wk * pc;
      G uxf = wk * uxc;
      G uyf = wk * uyc;
      G tf = wk * tc;
      // fp64: weights, stencil ids and the members past the compact stencil in batches of four
      // (those from memory, the compact ones staged); ref: weights in batches of eight, every
      // member staged.  Sums in stencil order either way.
      if constexpr (!kCompact) {
        for (int ci0 = 0; ci0 < nS; ci0 += 8) {
          S wb[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) wb[u] = (ci0 + u < nS) ? w[(size_t)(ci0 + u + 1) * ldc] : S(0);
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            if (ci0 + u < nS) {
              const V4<S> v = sv[(ci0 + u) * B + t];
              pf += wb[u] * v.x;
              uxf += wb[u] * v.y;
              uyf += wb[u] * v.z;
              tf += wb[u] * v.w;
            }
          }
        }
      } else
      for (int ci0 = 0; ci0 < nS; ci0 += 4) {
        S wb[4];
        int jj[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int ci = ci0 + u;
          wb[u] = ci < nS ? w[(size_t)(ci + 1) * ldc] : S(0);
          jj[u] = (ci < nS && ci >= nM) ? a.sten[ci * ldc + c] : c;
        }
        V4<WT> wv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) wv[u] = a.W[jj[u]];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int ci = ci0 + u;
          if (ci < nS) {
            const V4<S> v = ci < nM ? sv[ci * B + t] : V4<S>{(S)wv[u].x, (S)wv[u].y, (S)wv[u].z, (S)wv[u].w};
            pf += wb[u] * v.x;
            uxf += wb[u] * v.y;
            uyf += wb[u] * v.z;
            tf += wb[u] * v.w;
          }
        }
      }
      const S pnb = sv[fi * B + t].x;
      S phif;
      V4<G> o;
      limiter_process(lp, phif, pc, pMax, pMin, gPx, gPy, dx, dy);
      o.x = pick<P>(fab(pMax - pMin) >= SMALL, fab(pMax - pMin) < SMALL, pf, phif);
      notTrouble = phif > S(0);
      smooth = fmx(smooth, fab((S(1) - fraction) * pc + fraction * pnb - phif) / deltaR + (pf <= S(0)) * AFAR_LIT(S, 1e20) +
                               (phif <= S(0)) * AFAR_LIT(S, 1e20));
      limiter_process(lux, phif, uxc, uxMax, uxMin, gUxx, gUyx, dx, dy);
      o.y = pick<P>(fab(uxMax - uxMin) >= SMALL, fab(uxMax - uxMin) < SMALL, uxf, phif);
      limiter_process(luy, phif, uyc, uyMax, uyMin, gUxy, gUyy, dx, dy);
      o.z = pick<P>(fab(uyMax - uyMin) >= SMALL, fab(uyMax - uyMin) < SMALL, uyf, phif);
      limiter_process(lt, phif, tc, tMax, tMin, gTx, gTy, dx, dy);
      o.w = pick<P>(fab(tMax - tMin) >= SMALL, fab(tMax - tMin) < SMALL, tf, phif);
      notTrouble = phif > S(0);
      a.fv[2 * f + isNei] = o;
    }
    L.x = fmx(lp, S(0)) * notTrouble;
    L.y = fmx(lux, S(0)) * notTrouble;
    L.z = fmx(luy, S(0)) * notTrouble;
    L.w = fmx(lt, S(0)) * notTrouble;
    smooth = smooth / (S(0.5) * (pMax + pMin) * notTrouble + VSMALL);
    flag0 = (smooth > S(1));
  }
  a.lim[c] = L;
  a.si[2 * c] = flag0;
}

// Limiter maps (reference cudaLimiter.h:14-32)
template <class S>
__device__ __forceinline__ S to_bj(const S y) {
  return fmn(S(2) * y, S(1));
}
template <class S>
__device__ __forceinline__ S to_venkat(const S y) {
  return fmn((y * y + y + AFAR_LIT(S, 1e-10)) / (y * y + S(0.5) + S(0.5) * y + AFAR_LIT(S, 1e-10)), S(1));
}

// BVDindicator (reference cudaLimiter.h:319-464): stencil flag counts, BVD test on T, final
// switch type, limiter transform.
template <class P>
__device__ __forceinline__ void bvd_body(const StageArgs<P>& a, const int blk) {
  using S = typename P::S;
  using G = typename P::G;
  const int c = blk * blockDim.x + threadIdx.x;
  if (c >= a.Nc) return;
  const int ldc = a.ldc;
  const int nS = a.nS[c], nM = a.nM[c];
  int8_t shockType = a.si[2 * c];
  int8_t shockTypeExt = shockType;
  // troubled-cell flags of the stencil, eight index loads then eight flag loads at a time
  for (int i0 = 0; i0 < nS; i0 += 8) {
    int j[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) j[u] = (i0 + u < nS) ? a.sten[(i0 + u) * ldc + c] : c;
    int8_t fl[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) fl[u] = a.si[2 * j[u]];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int ci = i0 + u;
      if (ci < nM) {
        shockType += fl[u];
        shockTypeExt = shockType;
      } else if (ci < nS) {
        shockTypeExt += fl[u];
      }
    }
  }

  const S tc = (S)a.W[c].w;
  const V4<G> g1 = a.grad[2 * c + 1];
  const G gTx = g1.z, gTy = g1.w;
  V4<S> L = a.lim[c];
  int bvdType = 0, bfaces = 0;
  for (int fi = 0; fi < nM; ++fi) {
    int f = a.cf[fi * ldc + c];
    const bool isNei = (f < 0);
    f = abs(f) - 1;
    if (f >= a.Nf) {
      bfaces += 1;
      if (bfaces >= 2) {  // corner cell: low order
        bvdType = 1;
        break;
      }
      continue;
    }
    const V2<G> d = a.sg[fi * ldc + c];
    const G tfOwn = a.fv[2 * f].w;
    const G tfNei = a.fv[2 * f + 1].w;
    const G tfCur = pick<P>(isNei, !isNei, tfNei, tfOwn);
    const G tfOther = pick<P>(!isNei, isNei, tfNei, tfOwn);
    const G lim = to_bj(L.w);
    const G tfTVD = tc + lim * (gTx * d.x + gTy * d.y);
    const int typeval = fab(tfTVD - tfOther) < AFAR_LIT(S, 0.5) * fab(tfCur - tfOther);
    const int notFlat = fab(tfCur - tfOther) > AFAR_LIT(S, 1e-10);
    const int limited = (lim < AFAR_LIT(S, 0.9)) + (shockTypeExt > 0);
    bvdType = max(bvdType, notFlat * limited * typeval);
  }
  const int finalType = (shockType > 0) * (shockTypeExt > 1) * (-2) + (bvdType > 0);
  a.si[2 * c + 1] = (int8_t)finalType;
  const bool isShock = finalType < 0;
  if constexpr (P::exact_blend) {  // the reference's blend evaluates both maps
    L.x = pick<P>(isShock, !isShock, to_venkat(L.x), to_bj(L.x));
    L.y = pick<P>(isShock, !isShock, to_venkat(L.y), to_bj(L.y));
    L.z = pick<P>(isShock, !isShock, to_venkat(L.z), to_bj(L.z));
    L.w = pick<P>(isShock, !isShock, to_venkat(L.w), to_bj(L.w));
  } else if (isShock) {  // only the map that applies: Venkatakrishnan's has a division
    L.x = to_venkat(L.x);
    L.y = to_venkat(L.y);
    L.z = to_venkat(L.z);
    L.w = to_venkat(L.w);
  } else {
    L.x = to_bj(L.x);
    L.y = to_bj(L.y);
    L.z = to_bj(L.z);
    L.w = to_bj(L.w);
  }
  a.lim[c] = L;
}

// The mixed policy's FP32 Courant estimate of one internal face (setDeltaT, reference
// cudaFieldOperation.h:140-157): dt = CFL deltaR |Sf| / ((1-w)|U_o.Sf| + w|U_n.Sf| + c |Sf|),
// c = sqrt(gamma R ((1-w) T_o + w T_n)).  Every rounding is written out, so the fused stage-1 flux
// and the separate pass (afar_adjustTimeStep) give the same bits wherever the compiler places them.
__device__ __forceinline__ float courant_den_f32(const float fraction, const float magSf, const float Sfx,
                                                 const float Sfy, const V4<float>& Wo, const V4<float>& Wn,
                                                 const float gRf) {
  const float w0 = __fadd_rn(1.f, -fraction);
  const float unL = fabsf(__fmaf_rn(Wo.y, Sfx, __fmul_rn(Wo.z, Sfy)));
  const float unR = fabsf(__fmaf_rn(Wn.y, Sfx, __fmul_rn(Wn.z, Sfy)));
  const float c = __fsqrt_rn(__fmul_rn(gRf, __fmaf_rn(w0, Wo.w, __fmul_rn(fraction, Wn.w))));
  return __fmaf_rn(c, magSf, __fmaf_rn(w0, unL, __fmul_rn(fraction, unR)));
}
__device__ __forceinline__ float courant_dt_f32(const float cfl, const float deltaR, const float magSf,
                                                const float den) {
  return __fdiv_rn(__fmul_rn(__fmul_rn(cfl, deltaR), magSf), den);
}

// minimizeDeltaValue (reference cudaRiemannSolver.h:7-14)
template <class D, class G>
__device__ __forceinline__ D min_delta(const G l, const G r, const G lT, const G rT) {
  D d = fab(r - l);
  d = fmn((G)(d), fab(r - lT));
  d = fmn((G)(d), fab(rT - l));
  d = fmn((G)(d), fab(rT - lT));
  d = (r >= l) * d - (r < l) * d;
  return d;
}

// KFVSFlux (reference cudaRiemannSolver.h:16-68): adds (kinetic flux - central) so the face
// carries the kinetic flux-vector-splitting flux.
template <class D, class RC, class G>
__device__ __forceinline__ void kfvs_flux(G& rhoFlux, G& rhoUxFlux, G& rhoUyFlux, G& rhoEFlux, const D& rhoL,
                                          const D& rhoR, const D& pL, const D& pR, const D& uxL, const D& uxR,
                                          const D& uyL, const D& uyR, const D& tL, const D& tR, const RC& R,
                                          const RC& Cv, const D magSf, const D Sfx, const D Sfy) {
  const D nfx = Sfx / magSf;
  const D nfy = Sfy / magSf;
  const D uLl = uxL * nfx + uyL * nfy;
  const D vLl = uyL * nfx - uxL * nfy;
  const D uRl = uxR * nfx + uyR * nfy;
  const D vRl = uyR * nfx - uxR * nfy;
  const D lamL = D(0.5) * rhoL / pL;
  const D lamR = D(0.5) * rhoR / pR;
  // the reference writes pi as the float literal 3.141593f; the FP64 policy uses pi itself
  const D PI = std::is_same<D, float>::value ? (D)3.141593f : (D)3.14159265358979323846;
  const D m0p = D(0.5) * erfc_(-sqr_(lamL) * uLl);
  const D m1p = uLl * m0p + D(0.5) * exp_(-lamL * uLl * uLl) / (sqr_(PI * lamL));
  const D m2p = uLl * m1p + D(0.5) * m0p / lamL;
  const D m3p = uLl * m2p + m1p / lamL;
  const D m0n = D(0.5) * erfc_(sqr_(lamR) * uRl);
  const D m1n = uRl * m0n - D(0.5) * exp_(-lamR * uRl * uRl) / (sqr_(PI * lamR));
  const D m2n = uRl * m1n + D(0.5) * m0n / lamR;
  const D m3n = uRl * m2n + m1n / lamR;
  const D& mvL = vLl;
  const D& mvR = vRl;
  const D K = D(2) * Cv / R - D(2);
  const D trho = rhoL * m1p + rhoR * m1n;
  const D trhoUx = rhoL * m2p + rhoR * m2n;
  const D trhoUy = rhoL * m1p * mvL + rhoR * m1n * mvR;
  const D trhoE = D(0.5) * rhoL * (m3p + m1p * (vLl * mvL + D(0.5) / lamL) + m1p * K * D(0.5) / lamL) +
                  D(0.5) * rhoR * (m3n + m1n * (vRl * mvR + D(0.5) / lamR) + m1n * K * D(0.5) / lamR);
  rhoUxFlux += trhoUx * Sfx - trhoUy * Sfy - D(0.5) * ((D)(rhoFlux)*uxL + pL * Sfx) - D(0.5) * ((D)(rhoFlux)*uxR + pR * Sfx);
  rhoUyFlux += trhoUx * Sfy + trhoUy * Sfx - D(0.5) * ((D)(rhoFlux)*uyL + pL * Sfy) - D(0.5) * ((D)(rhoFlux)*uyR + pR * Sfy);
  rhoEFlux += trhoE * magSf - D(0.5) * (D)(rhoFlux) * (Cv * tL + D(0.5) * (uxL * uxL + uyL * uyL) + pL / rhoL) -
              D(0.5) * (D)(rhoFlux) * (Cv * tR + D(0.5) * (uxR * uxR + uyR * uyR) + pR / rhoR);
  rhoFlux += trho * magSf - D(0.5) * rhoL * (uxL * Sfx + uyL * Sfy) - D(0.5) * rhoR * (uxR * Sfx + uyR * Sfy);
}

// RoeFlux (reference cudaRiemannSolver.h:71-136): Roe dissipation with a Harten-type entropy fix.
template <class D, class RC, class G>
__device__ __forceinline__ void roe_flux(G& rhoFlux, G& rhoUxFlux, G& rhoUyFlux, G& rhoEFlux, const D& rhoL,
                                         const D& rhoR, const D& pL, const D& pR, const D& uxL, const D& uxR,
                                         const D& uyL, const D& uyR, const D& tL, const D& tR, const D& deltaP,
                                         const D& deltaRho, const RC& R, const RC& Cv, const D magSf, const D Sfx,
                                         const D Sfy) {
  const D gamma = (Cv + R) / Cv;
  const D nfx = Sfx / magSf;
  const D nfy = Sfy / magSf;
  const D cvL = uxL * nfx + uyL * nfy;
  const D cvR = uxR * nfx + uyR * nfy;
  const D hL = Cv * tL + D(0.5) * (uxL * uxL + uyL * uyL) + pL / rhoL;
  const D hR = Cv * tR + D(0.5) * (uxR * uxR + uyR * uyR) + pR / rhoR;
  const D tiny = AFAR_LIT(D, 1e-20);
  const D rhoT = sqr_(fmx(rhoL * rhoR, tiny));
  const D wL = sqr_(fmx(rhoL, tiny)) / (sqr_(fmx(rhoL, tiny)) + sqr_(fmx(rhoR, tiny)));
  const D wR = D(1) - wL;
  const D uxT = uxL * wL + uxR * wR;
  const D uyT = uyL * wL + uyR * wR;
  const D hT = hL * wL + hR * wR;
  const D q2 = uxT * uxT + uyT * uyT;
  const D cT = sqr_(fmx((gamma - D(1)) * (hT - D(0.5) * q2), tiny));
  const D cvT = uxT * nfx + uyT * nfy;
  const D dUx = uxR - uxL;
  const D dUy = uyR - uyL;
  const D dCv = dUx * nfx + dUy * nfy;
  const D r1 = (deltaP - rhoT * cT * dCv) / (D(2) * cT * cT);
  const D r2 = deltaRho - deltaP / (cT * cT);
  const D r3 = (deltaP + rhoT * cT * dCv) / (D(2) * cT * cT);
  const D& UL = cvL;
  const D& UR = cvR;
  const D cL = sqr_(fmx((gamma - D(1)) * (hL - D(0.5) * (uxL * uxL + uyL * uyL)), tiny));
  const D cR = sqr_(fmx((gamma - D(1)) * (hR - D(0.5) * (uxR * uxR + uyR * uyR)), tiny));
  const D eps0 = AFAR_LIT(D, 1e-30);
  D eps = D(2) * fmx(D(0), (UR - cR) - (UL - cL));
  D l1 = fab(cvT - cT);
  l1 = (l1 >= eps) * l1 + (l1 < eps) * ((l1 * l1 + eps * eps) / (D(2) * eps + eps0));
  eps = D(2) * fmx(D(0), UR - UL);
  D l2 = fab(cvT);
  l2 = (l2 >= eps) * l2 + (l2 < eps) * ((l2 * l2 + eps * eps) / (D(2) * eps + eps0));
  eps = D(2) * fmx(D(0), (UR + cR) - (UL + cL));
  D l3 = fab(cvT + cT);
  l3 = (l3 >= eps) * l3 + (l3 < eps) * ((l3 * l3 + eps * eps) / (D(2) * eps + eps0));
  rhoFlux -= D(0.5) * (l1 * r1 + l2 * r2 + l3 * r3) * magSf;
  rhoUxFlux -= D(0.5) * (l1 * r1 * (uxT - cT * nfx) + l2 * (r2 * uxT + rhoT * (dUx - dCv * nfx)) + l3 * r3 * (uxT + cT * nfx)) * magSf;
  rhoUyFlux -= D(0.5) * (l1 * r1 * (uyT - cT * nfy) + l2 * (r2 * uyT + rhoT * (dUy - dCv * nfy)) + l3 * r3 * (uyT + cT * nfy)) * magSf;
  rhoEFlux -= D(0.5) *
              (l1 * r1 * (hT - cT * cvT) + l2 * (r2 * D(0.5) * q2 + rhoT * (uxT * dUx + uyT * dUy - cvT * dCv)) +
               l3 * r3 * (hT + cT * cvT)) *
              magSf;
}

// ---------------------------------------------------------------- dissipation, fp64 and mixed
// The same Roe and KFVS dissipation for the policies without bit parity, with their divisions
// folded: p/rho as R T (the state's own equation of state), one reciprocal of magSf (precomputed
// per face), of c^2 and of lambda, gamma and K computed once on the host, and the entropy fix's
// division only on the faces that need it.  Equal to the reference's expressions up to rounding.
__device__ __forceinline__ double fdiv(const double a, const double b) { return a / b; }
__device__ __forceinline__ float fdiv(const float a, const float b) { return __fdividef(a, b); }
__device__ __forceinline__ double rsqrt_(const double a) { return rsqrt(a); }
__device__ __forceinline__ float rsqrt_(const float a) { return rsqrtf(a); }

template <class D>
__device__ __forceinline__ void entropy_fix(D& l, const D eps) {
  if (l < eps) l = fdiv(l * l + eps * eps, D(2) * eps + AFAR_LIT(D, 1e-30));
}

template <class D>
__device__ __forceinline__ void roe_flux_fast(D& rhoFlux, D& rhoUxFlux, D& rhoUyFlux, D& rhoEFlux, const D rhoL,
                                              const D rhoR, const D uxL, const D uxR, const D uyL, const D uyR,
                                              const D tL, const D tR, const D deltaP, const D deltaRho, const D R,
                                              const D Cv, const D gamma, const D magSf, const D nfx, const D nfy) {
  const D cvL = uxL * nfx + uyL * nfy;
  const D cvR = uxR * nfx + uyR * nfy;
  const D kL = D(0.5) * (uxL * uxL + uyL * uyL), kR = D(0.5) * (uxR * uxR + uyR * uyR);
  const D hL = Cv * tL + kL + R * tL;
  const D hR = Cv * tR + kR + R * tR;
  const D tiny = AFAR_LIT(D, 1e-20);
  const D sL = sqr_(fmx(rhoL, tiny)), sR = sqr_(fmx(rhoR, tiny));
  const D rhoT = sL * sR;  // sqrt(rhoL rhoR) from the two roots the weights need anyway
  const D wL = fdiv(sL, sL + sR);
  const D wR = D(1) - wL;
  const D uxT = uxL * wL + uxR * wR;
  const D uyT = uyL * wL + uyR * wR;
  const D hT = hL * wL + hR * wR;
  const D q2 = uxT * uxT + uyT * uyT;
  const D cT2 = fmx((gamma - D(1)) * (hT - D(0.5) * q2), tiny);
  const D rcT = rsq_(cT2);  // 1/cT: the speed and 1/cT^2 from one reciprocal root
  const D cT = cT2 * rcT;
  const D ic2 = rcT * rcT;
  const D cvT = uxT * nfx + uyT * nfy;
  const D dUx = uxR - uxL;
  const D dUy = uyR - uyL;
  const D dCv = dUx * nfx + dUy * nfy;
  const D r1 = (deltaP - rhoT * cT * dCv) * (D(0.5) * ic2);
  const D r2 = deltaRho - deltaP * ic2;
  const D r3 = (deltaP + rhoT * cT * dCv) * (D(0.5) * ic2);
  const D cL = sqr_(fmx((gamma - D(1)) * (hL - kL), tiny));
  const D cR = sqr_(fmx((gamma - D(1)) * (hR - kR), tiny));
  D l1 = fab(cvT - cT), l2 = fab(cvT), l3 = fab(cvT + cT);
  entropy_fix(l1, D(2) * fmx(D(0), (cvR - cR) - (cvL - cL)));
  entropy_fix(l2, D(2) * fmx(D(0), cvR - cvL));
  entropy_fix(l3, D(2) * fmx(D(0), (cvR + cR) - (cvL + cL)));
  rhoFlux -= D(0.5) * (l1 * r1 + l2 * r2 + l3 * r3) * magSf;
  rhoUxFlux -= D(0.5) * (l1 * r1 * (uxT - cT * nfx) + l2 * (r2 * uxT + rhoT * (dUx - dCv * nfx)) + l3 * r3 * (uxT + cT * nfx)) * magSf;
  rhoUyFlux -= D(0.5) * (l1 * r1 * (uyT - cT * nfy) + l2 * (r2 * uyT + rhoT * (dUy - dCv * nfy)) + l3 * r3 * (uyT + cT * nfy)) * magSf;
  rhoEFlux -= D(0.5) *
              (l1 * r1 * (hT - cT * cvT) + l2 * (r2 * D(0.5) * q2 + rhoT * (uxT * dUx + uyT * dUy - cvT * dCv)) +
               l3 * r3 * (hT + cT * cvT)) *
              magSf;
}

template <class D>
__device__ __forceinline__ void kfvs_flux_fast(D& rhoFlux, D& rhoUxFlux, D& rhoUyFlux, D& rhoEFlux, const D rhoL,
                                               const D rhoR, const D pL, const D pR, const D uxL, const D uxR,
                                               const D uyL, const D uyR, const D tL, const D tR, const D R, const D Cv,
                                               const D K, const D magSf, const D nfx, const D nfy) {
  const D Sfx = nfx * magSf, Sfy = nfy * magSf;
  const D uLl = uxL * nfx + uyL * nfy;
  const D vLl = uyL * nfx - uxL * nfy;
  const D uRl = uxR * nfx + uyR * nfy;
  const D vRl = uyR * nfx - uxR * nfy;
  const D ilamL = D(2) * R * tL, ilamR = D(2) * R * tR;  // 1/lambda = 2 p / rho
  const D lamL = fdiv(D(1), ilamL), lamR = fdiv(D(1), ilamR);
  const D PI = std::is_same<D, float>::value ? (D)3.141593f : (D)3.14159265358979323846;
  const D m0p = D(0.5) * erfc_(-sqr_(lamL) * uLl);
  const D m1p = uLl * m0p + D(0.5) * exp_(-lamL * uLl * uLl) * rsqrt_(PI * lamL);
  const D m2p = uLl * m1p + D(0.5) * m0p * ilamL;
  const D m3p = uLl * m2p + m1p * ilamL;
  const D m0n = D(0.5) * erfc_(sqr_(lamR) * uRl);
  const D m1n = uRl * m0n - D(0.5) * exp_(-lamR * uRl * uRl) * rsqrt_(PI * lamR);
  const D m2n = uRl * m1n + D(0.5) * m0n * ilamR;
  const D m3n = uRl * m2n + m1n * ilamR;
  const D trho = rhoL * m1p + rhoR * m1n;
  const D trhoUx = rhoL * m2p + rhoR * m2n;
  const D trhoUy = rhoL * m1p * vLl + rhoR * m1n * vRl;
  const D trhoE = D(0.5) * rhoL * (m3p + m1p * (vLl * vLl + D(0.5) * ilamL) + m1p * K * D(0.5) * ilamL) +
                  D(0.5) * rhoR * (m3n + m1n * (vRl * vRl + D(0.5) * ilamR) + m1n * K * D(0.5) * ilamR);
  rhoUxFlux += trhoUx * Sfx - trhoUy * Sfy - D(0.5) * (rhoFlux * uxL + pL * Sfx) - D(0.5) * (rhoFlux * uxR + pR * Sfx);
  rhoUyFlux += trhoUx * Sfy + trhoUy * Sfx - D(0.5) * (rhoFlux * uyL + pL * Sfy) - D(0.5) * (rhoFlux * uyR + pR * Sfy);
  rhoEFlux += trhoE * magSf - D(0.5) * rhoFlux * (Cv * tL + D(0.5) * (uxL * uxL + uyL * uyL) + R * tL) -
              D(0.5) * rhoFlux * (Cv * tR + D(0.5) * (uxR * uxR + uyR * uyR) + R * tR);
  rhoFlux += trho * magSf - D(0.5) * rhoL * (uxL * Sfx + uyL * Sfy) - D(0.5) * rhoR * (uxR * Sfx + uyR * Sfy);
}

// ---------------------------------------------------------------- ref policy: face flux
// The ref policy's face flux reproduces the reference kernel's results bit for bit.  Two things
// besides the arithmetic itself decide that, both established by comparing with the reference
// kernels' results on the parity meshes (never by reading compiled code):
//  * nvcc contracts plain a*b + c expressions into fused multiply-adds in ways that depend on the
//    surrounding code, so every double-precision rounding of the state selection and the central
//    flux is written out (__fma_rn / __dmul_rn / __dadd_rn) in the pattern the reference's build
//    produces (identified on 24,300 faces of a mixed quad/triangle Riemann mesh, every candidate
//    rounding evaluated exactly);
//  * the float Roe/KFVS dissipation rounds like the reference's only when it is compiled as a
//    function of its own that takes its inputs by reference and is called through a pointer: inlined,
//    called directly, or taking its inputs by value, its float expressions round differently on a
//    few hundred flux entries per mesh (a few ulp of float).
// A blend c1*a + c2*b with c in {0, 1} is exact either way; it keeps the reference's propagation of
// a non-finite unused operand.

// One side of an internal face: the limited linear (TVD) state at the face centre, and the state
// the flux uses (the O3 face value, or the TVD state where the cell's switch asks for it), with
// p/(R T) of both; reference cudaRiemannSolver.h:190-216.
struct RefSide {
  double p, ux, uy, T, rho;  // the state the flux uses
  double pT, rhoT;           // pressure and density of the TVD state
};
__device__ __forceinline__ double ref_tvd(const double w, const float lim, const double ga, const double gb,
                                          const double dx, const double dy) {
  return __fma_rn((double)lim, __fma_rn(ga, dx, __dmul_rn(gb, dy)), w);  // w + lim (ga dx + gb dy)
}
__device__ __forceinline__ double ref_blend(const bool tvd, const double o3, const double t) {
  return __dadd_rn(__dmul_rn((double)(1 - tvd), o3), __dmul_rn((double)tvd, t));
}
__device__ __forceinline__ RefSide ref_face_side(const StageArgs<PolicyRef>& a, const int c, const int slot,
                                                 const double dx, const double dy, const bool tvd) {
  const V4<double> w = a.W[c];
  const V4<double> g0 = a.grad[2 * c], g1 = a.grad[2 * c + 1];  // (px py uxx uxy), (uyx uyy tx ty)
  const V4<float> lm = a.lim[c];
  const V4<double> o3 = a.fv[slot];
  const double R = a.R;
  const double pT = ref_tvd(w.x, lm.x, g0.x, g0.y, dx, dy);
  const double uxT = ref_tvd(w.y, lm.y, g0.z, g1.x, dx, dy);
  const double uyT = ref_tvd(w.z, lm.z, g0.w, g1.y, dx, dy);
  const double tT = ref_tvd(w.w, lm.w, g1.z, g1.w, dx, dy);
  RefSide s;
  s.pT = pT;
  s.rhoT = pT / __dmul_rn(R, tT);
  s.p = ref_blend(tvd, o3.x, pT);
  s.ux = ref_blend(tvd, o3.y, uxT);
  s.uy = ref_blend(tvd, o3.z, uyT);
  s.T = ref_blend(tvd, o3.w, tT);
  s.rho = s.p / __dmul_rn(R, s.T);
  return s;
}
// Cv T + |u|^2 / 2 + p / rho of a side (its total enthalpy per unit mass)
__device__ __forceinline__ double ref_enthalpy(const RefSide& s, const double Cv) {
  return __dadd_rn(__dadd_rn(__dmul_rn(Cv, s.T), __dmul_rn(0.5, __fma_rn(s.ux, s.ux, __dmul_rn(s.uy, s.uy)))),
                   s.p / s.rho);
}

// The float dissipation of the ref policy: adds the Roe dissipation, or replaces the central flux
// by the KFVS flux, in the four double flux components (reference cudaRiemannSolver.h:16-136).
using RefDissipation = void (*)(double&, double&, double&, double&, const float&, const float&, const float&,
                                const float&, const float&, const float&, const float&, const float&, const float&,
                                const float&, const float&, const float&, const double&, const double&, const float,
                                const float, const float);
__device__ __noinline__ void ref_roe(double& rhoFlux, double& rhoUxFlux, double& rhoUyFlux, double& rhoEFlux,
                                     const float& rhoL, const float& rhoR, const float& pL, const float& pR,
                                     const float& uxL, const float& uxR, const float& uyL, const float& uyR,
                                     const float& tL, const float& tR, const float& dP, const float& dRho,
                                     const double& R, const double& Cv, const float magSf, const float Sfx,
                                     const float Sfy) {
  roe_flux<float, double, double>(rhoFlux, rhoUxFlux, rhoUyFlux, rhoEFlux, rhoL, rhoR, pL, pR, uxL, uxR, uyL, uyR, tL,
                                  tR, dP, dRho, R, Cv, magSf, Sfx, Sfy);
}
__device__ __noinline__ void ref_kfvs(double& rhoFlux, double& rhoUxFlux, double& rhoUyFlux, double& rhoEFlux,
                                      const float& rhoL, const float& rhoR, const float& pL, const float& pR,
                                      const float& uxL, const float& uxR, const float& uyL, const float& uyR,
                                      const float& tL, const float& tR, const float&, const float&,
                                      const double& R, const double& Cv, const float magSf, const float Sfx,
                                      const float Sfy) {
  kfvs_flux<float, double, double>(rhoFlux, rhoUxFlux, rhoUyFlux, rhoEFlux, rhoL, rhoR, pL, pR, uxL, uxR, uyL, uyR, tL,
                                   tR, R, Cv, magSf, Sfx, Sfy);
}

// evaluateFlux of internal face f under the ref policy (reference cudaRiemannSolver.h:171-251):
// both sides' states, the minimised jumps of p and rho, the central flux in double, then the float
// Roe dissipation, or the KFVS flux where either cell is a shock cell.
__device__ __forceinline__ void flux_ref_face(const StageArgs<PolicyRef>& a, const int f) {
  const int2 on = a.on[f];
  const V4<double> d = a.fd[f];   // face centre - owner centre, face centre - neighbour centre
  const V4<double> sf = a.fs[f];  // Sfx, Sfy, |Sf|
  const int8_t swL = a.si[2 * on.x + 1], swR = a.si[2 * on.y + 1];
  const RefSide L = ref_face_side(a, on.x, 2 * f, d.x, d.y, swL != 0);
  const RefSide Rs = ref_face_side(a, on.y, 2 * f + 1, d.z, d.w, swR != 0);
  const double Sfx = sf.x, Sfy = sf.y, magSf = sf.z, Cv = a.Cv, R = a.R;
  const float dP = min_delta<float, double>(L.p, Rs.p, L.pT, Rs.pT);
  const float dRho = min_delta<float, double>(L.rho, Rs.rho, L.rhoT, Rs.rhoT);
  // central flux: the mean of the two sides' Euler fluxes through Sf
  double F0, F1, F2, F3;
  const double unL = __fma_rn(L.ux, Sfx, __dmul_rn(L.uy, Sfy)), unR = __fma_rn(Rs.ux, Sfx, __dmul_rn(Rs.uy, Sfy));
  F0 = __fma_rn(__dmul_rn(0.5, L.rho), unL, __dmul_rn(__dmul_rn(0.5, Rs.rho), unR));
  F1 = __dadd_rn(__dmul_rn(0.5, __fma_rn(L.p, Sfx, __dmul_rn(F0, L.ux))),
                 __dmul_rn(0.5, __fma_rn(Rs.p, Sfx, __dmul_rn(F0, Rs.ux))));
  F2 = __dadd_rn(__dmul_rn(0.5, __fma_rn(L.p, Sfy, __dmul_rn(F0, L.uy))),
                 __dmul_rn(0.5, __fma_rn(Rs.p, Sfy, __dmul_rn(F0, Rs.uy))));
  const double half = __dmul_rn(0.5, F0);
  F3 = __fma_rn(half, ref_enthalpy(L, Cv), __dmul_rn(half, ref_enthalpy(Rs, Cv)));
  // the dissipation sees the states, face vector and jumps as floats; R and Cv stay double
  const float rhoL = L.rho, rhoR = Rs.rho, pL = L.p, pR = Rs.p, uxL = L.ux, uxR = Rs.ux, uyL = L.uy, uyR = Rs.uy,
              tL = L.T, tR = Rs.T;
  const RefDissipation diss = (swL < 0 || swR < 0) ? ref_kfvs : ref_roe;
  diss(F0, F1, F2, F3, rhoL, rhoR, pL, pR, uxL, uxR, uyL, uyR, tL, tR, dP, dRho, R, Cv, (float)magSf, (float)Sfx,
       (float)Sfy);
  a.flux[f] = V4<double>{F0, F1, F2, F3};
}

// evaluateFlux (reference cudaRiemannSolver.h:155-271): one thread per internal face, then one per
// boundary face (ids Nf..Nf+Nb-1; the reference's grid covers boundary faces b < 128*ceil(Nf/128)
// only, which holds on every mesh with Nf >= Nb).  DT: also reduce the CFL step of the reference's
// setDeltaT (cudaFieldOperation.h:124-180) from the state at the start of the step.
template <class P, bool DT>
__device__ __forceinline__ void flux_body(const StageArgs<P>& a, const int blk) {
  using S = typename P::S;
  using G = typename P::G;
  using D = typename P::D;
  using RC = typename P::RC;
  constexpr bool kF32 = std::is_same<G, float>::value;  // mixed: no per-thread FP64 at all
  const int id = blk * blockDim.x + threadIdx.x;
  // the Courant step: mixed estimates it in FP32 from block constants read once by thread 0
  __shared__ float s_cfl;
  __shared__ int s_cfl_step;
  if constexpr (DT && kF32) {
    if (threadIdx.x == 0) {
      s_cfl_step = !(a.ctl->dt_fixed > 0.0);
      s_cfl = (float)a.ctl->cfl;
    }
    __syncthreads();
  }
  double dtf = 1e5;
  float dtf32 = 1e5f;
  if (id < a.Nf) {
    if constexpr (P::id == PolicyRef::id) {
      static_assert(!DT, "under the ref policy the Courant step is a kernel of its own, as in the reference");
      flux_ref_face(a, id);
    } else {
      const int2 on = a.on[id];
      const int own = on.x, nei = on.y;
      const V4<G> fd = a.fd[id];
      const G dxL = fd.x, dyL = fd.y, dxR = fd.z, dyR = fd.w;
      const int8_t sL = a.si[2 * own + 1], sR = a.si[2 * nei + 1];
      const bool tvdL = sL != 0, tvdR = sR != 0;
      const bool isShock = sL < 0 || sR < 0;
      const V4<G> fs = a.fs[id];
      const G Sfx = fs.x, Sfy = fs.y, magSf = fs.z;
      G R, Cv, iR, gam;
      if constexpr (kF32) {
        R = a.Rf;
        Cv = a.Cvf;
        iR = a.invRf;
        gam = a.gm1f + 1.f;
      } else {
        R = (G)a.R;
        Cv = (G)a.Cv;
        iR = (G)a.invR;
        gam = (G)a.gamma;
      }
      const V4<typename P::W> Wo = a.W[own], Wn = a.W[nei];
      const V4<G> go0 = a.grad[2 * own], go1 = a.grad[2 * own + 1];
      const V4<G> gn0 = a.grad[2 * nei], gn1 = a.grad[2 * nei + 1];
      const V4<S> lo = a.lim[own], ln = a.lim[nei];
      const V4<G> fo = a.fv[2 * id], fn = a.fv[2 * id + 1];
      G rhoFlux, rhoUxFlux, rhoUyFlux, rhoEFlux;
      D pLf, uxLf, uyLf, tLf, rhoLf, pRf, uxRf, uyRf, tRf, rhoRf, dP, dRho;
      {
        const G pLT = (G)Wo.x + lo.x * (go0.x * dxL + go0.y * dyL);
        const G uxLT = (G)Wo.y + lo.y * (go0.z * dxL + go1.x * dyL);
        const G uyLT = (G)Wo.z + lo.z * (go0.w * dxL + go1.y * dyL);
        const G tLT = (G)Wo.w + lo.w * (go1.z * dxL + go1.w * dyL);
        const G pRT = (G)Wn.x + ln.x * (gn0.x * dxR + gn0.y * dyR);
        const G uxRT = (G)Wn.y + ln.y * (gn0.z * dxR + gn1.x * dyR);
        const G uyRT = (G)Wn.z + ln.z * (gn0.w * dxR + gn1.y * dyR);
        const G tRT = (G)Wn.w + ln.w * (gn1.z * dxR + gn1.w * dyR);
        const G pL = pick<P>(!tvdL, tvdL, fo.x, pLT);
        const G uxL = pick<P>(!tvdL, tvdL, fo.y, uxLT);
        const G uyL = pick<P>(!tvdL, tvdL, fo.z, uyLT);
        const G tL = pick<P>(!tvdL, tvdL, fo.w, tLT);
        const G pR = pick<P>(!tvdR, tvdR, fn.x, pRT);
        const G uxR = pick<P>(!tvdR, tvdR, fn.y, uxRT);
        const G uyR = pick<P>(!tvdR, tvdR, fn.z, uyRT);
        const G tR = pick<P>(!tvdR, tvdR, fn.w, tRT);
        G rhoLT, rhoRT, rhoL, rhoR;  // p / (R T) of the four states
        if constexpr (kF32) {
          rhoLT = fdiv(pLT * iR, tLT);
          rhoRT = fdiv(pRT * iR, tRT);
          rhoL = fdiv(pL * iR, tL);
          rhoR = fdiv(pR * iR, tR);
        } else {
          // FP64: the four reciprocal temperatures from one division (Montgomery's simultaneous
          // inversion, a few ulps from four divisions); a double division is among the dearest
          // operations of GB300's FP64 pipe, which bounds this kernel.  Temperatures stay far from
          // the range limits of double (their product of four neither overflows nor underflows).
          const G tt = tL * tR, ttT = tLT * tRT;
          const G inv = G(1) / (tt * ttT);
          const G itt = inv * ttT, ittT = inv * tt;  // 1/(tL tR), 1/(tLT tRT)
          rhoL = pL * iR * (itt * tR);
          rhoR = pR * iR * (itt * tL);
          rhoLT = pLT * iR * (ittT * tRT);
          rhoRT = pRT * iR * (ittT * tLT);
        }
        dP = min_delta<D, G>(pL, pR, pLT, pRT);
        dRho = min_delta<D, G>(rhoL, rhoR, rhoLT, rhoRT);
        const G h = G(0.5);
        rhoFlux = h * rhoL * (uxL * Sfx + uyL * Sfy) + h * rhoR * (uxR * Sfx + uyR * Sfy);
        rhoUxFlux = h * (rhoFlux * uxL + pL * Sfx) + h * (rhoFlux * uxR + pR * Sfx);
        rhoUyFlux = h * (rhoFlux * uyL + pL * Sfy) + h * (rhoFlux * uyR + pR * Sfy);
        rhoEFlux = h * rhoFlux * (Cv * tL + h * (uxL * uxL + uyL * uyL) + R * tL) +  // p/rho = R T
                   h * rhoFlux * (Cv * tR + h * (uxR * uxR + uyR * uyR) + R * tR);
        pLf = pL; uxLf = uxL; uyLf = uyL; tLf = tL; rhoLf = rhoL;
        pRf = pR; uxRf = uxR; uyRf = uyR; tRf = tR; rhoRf = rhoR;
      }
      static_assert(std::is_same<D, G>::value, "fp64 and mixed run the dissipation in their face-value type");
      const G nfx = Sfx * fs.w, nfy = Sfy * fs.w;  // fs.w = 1/|Sf| (setup)
      if (isShock)
        kfvs_flux_fast<G>(rhoFlux, rhoUxFlux, rhoUyFlux, rhoEFlux, rhoLf, rhoRf, pLf, pRf, uxLf, uxRf, uyLf, uyRf, tLf,
                          tRf, R, Cv, G(2) * Cv * iR - G(2), magSf, nfx, nfy);
      else
        roe_flux_fast<G>(rhoFlux, rhoUxFlux, rhoUyFlux, rhoEFlux, rhoLf, rhoRf, uxLf, uxRf, uyLf, uyRf, tLf, tRf, dP,
                         dRho, R, Cv, gam, magSf, nfx, nfy);
      a.flux[id] = V4<typename P::F>{(typename P::F)rhoFlux, (typename P::F)rhoUxFlux, (typename P::F)rhoUyFlux,
                                     (typename P::F)rhoEFlux};
      if constexpr (DT && kF32) {
        if (s_cfl_step) {  // setDeltaT, cudaFieldOperation.h:140-157, as an FP32 estimate
          const V2<float> g = a.dtgf[id];
          dtf32 = courant_dt_f32(s_cfl, g.x, magSf, courant_den_f32(g.y, magSf, Sfx, Sfy, Wo, Wn, a.gRf));
        }
      } else if (DT) {
        const StepCtl* ctl = a.ctl;
        if (!(ctl->dt_fixed > 0.0)) {  // setDeltaT, cudaFieldOperation.h:140-157
          const V2<double> g = a.dtg[id];
          const double deltaR = g.x, fraction = g.y;
          const double sfx = (double)Sfx, sfy = (double)Sfy, msf = (double)magSf;
          const double CFL = ctl->cfl, Rd = a.R, Cvd = a.Cv;
          dtf = CFL * deltaR * msf /
                ((1.0 - fraction) * fabs((double)Wo.y * sfx + (double)Wo.z * sfy) +
                 fraction * fabs((double)Wn.y * sfx + (double)Wn.z * sfy) +
                 sqrt((Rd / Cvd + 1.0) * Rd * ((1.0 - fraction) * (double)Wo.w + fraction * (double)Wn.w)) * msf);
        }
      }
    }
  } else if (id < a.Nf + a.Nb) {  // boundary faces, reference :254-270
    const int b = id - a.Nf;
    const V4<typename P::W> wb = a.W[a.Nc + b];
    const V4<G> fs = a.fs[id];
    const G Sfx = fs.x, Sfy = fs.y;
    G R, Cv;
    if constexpr (kF32) {
      R = a.Rf;
      Cv = a.Cvf;
    } else {
      R = (G)a.R;
      Cv = (G)a.Cv;
    }
    const G bp = wb.x, bUx = wb.y, bUy = wb.z, bT = wb.w;
    const G rho = bp / (R * bT);
    const G rhoFlux = rho * (bUx * Sfx + bUy * Sfy);
    a.flux[id] = V4<typename P::F>{(typename P::F)rhoFlux, (typename P::F)(rhoFlux * bUx + bp * Sfx),
                                   (typename P::F)(rhoFlux * bUy + bp * Sfy),
                                   (typename P::F)(rhoFlux * (Cv * bT + G(0.5) * (bUx * bUx + bUy * bUy) + bp / rho))};
  }
  if constexpr (DT && kF32) {
    // block min of the float estimates on their bit patterns (non-negative floats order like
    // them; NaN sorts above +inf), then one atomicMin per block on the double's bits
    unsigned v = (unsigned)__float_as_int(dtf32);
    if (!(dtf32 >= 0.f)) v = 0x7F800000u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned u = __shfl_xor_sync(0xffffffffu, v, o);
      v = u < v ? u : v;
    }
    __shared__ unsigned wmin32[8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) wmin32[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned m = wmin32[0];
      for (int k = 1; k < (int)(blockDim.x >> 5); ++k) m = wmin32[k] < m ? wmin32[k] : m;
      const float mf = __int_as_float((int)m);
      const unsigned long long bits =
          m >= 0x7F800000u ? 0x7FF0000000000000ull : (unsigned long long)__double_as_longlong((double)mf);
      atomicMin(&a.ctl->dt_bits, bits);
    }
  } else if (DT) {
    // block min (warp shuffles) then one atomicMin per block on the bit pattern; non-negative
    // doubles order like their bit patterns, and NaN patterns sort above +inf.
    unsigned long long v = (unsigned long long)__double_as_longlong(dtf);
    if (!(dtf >= 0.0)) v = 0x7FF0000000000000ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long u = __shfl_xor_sync(0xffffffffu, v, o);
      v = u < v ? u : v;
    }
    __shared__ unsigned long long wmin[8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) wmin[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned long long m = wmin[0];
      for (int k = 1; k < (int)(blockDim.x >> 5); ++k) m = wmin[k] < m ? wmin[k] : m;
      atomicMin(&a.ctl->dt_bits, m);
    }
  }
}

// Ghost state of boundary face b from its owner's state (reference cudaEulerBCs.h:45-95 and
// BCs/2D/<label>.h:4-10).
__device__ __forceinline__ V4<double> boundary_value(const int type, const V4<double> w, const V2<double> n) {
  switch (type) {
    case 0:  // constantTemperatureWallBoundary
      return V4<double>{w.x, 0.0, 0.0, 1.0};
    case 1:  // adiabaticWallBoundary
      return V4<double>{w.x, 0.0, 0.0, w.w};
    case 2:  // symmetryBoundary
      return V4<double>{w.x, w.y - (w.y * n.x + w.z * n.y) * n.x, w.z - (w.y * n.x + w.z * n.y) * n.y, w.w};
    case 3:  // fixedValueBoundary
      return V4<double>{1.0, 3.0, 0.0, 1.0};
    case 4:  // outletBoundary
      return w;
    case 5:  // fixedValue2Boundary
      return V4<double>{30.05945, 4.07795, 0.0, 5.97677};
    default:
      return w;
  }
}

// Error-free float addition (Knuth two-sum): s + e == a + b exactly.
__device__ __forceinline__ void two_sum(float& s, float& e, const float a, const float b) {
  s = a + b;
  const float bp = s - a;
  e = (a - (s - bp)) + (b - bp);
}

// The mixed policy's gather + update, with no FP64 arithmetic on the path (GB300's FP64 pipe is
// 1/53 of FP32): the residual of the float fluxes is summed error-free as a float pair, the
// conserved state U, Un is stored and combined as float pairs (DF4, ~48 bits), and the pressure is
// the float-pair difference rhoE - |rhoU|^2/(2 rho) (the cancellation at high Mach costs no
// precision), rounded once to float.  k = {beta3*dt, beta1 (hi, lo), beta2 (hi, lo)} of the stage.
template <class P>
__device__ __forceinline__ void update_mixed(const StageArgs<P>& a, const int c, const StageCoef& k,
                                             const int* s_go, const float* s_bdt) {
  const int ldc = a.ldc;
  const bool live = c < a.Nc;
  const int nM = live ? a.nM[c] : 0;
  float hi[4] = {0.f, 0.f, 0.f, 0.f}, lo[4] = {0.f, 0.f, 0.f, 0.f};
  constexpr int MB = 4;
  for (int f0 = 0; f0 < nM; f0 += MB) {  // the gather needs no step size: it overlaps thread 0's work
    int fid[MB];
#pragma unroll
    for (int u = 0; u < MB; ++u) fid[u] = (f0 + u < nM) ? a.cf[(f0 + u) * ldc + c] : 1;
    V4<float> fl[MB];
#pragma unroll
    for (int u = 0; u < MB; ++u) fl[u] = reinterpret_cast<const V4<float>*>(a.flux)[abs(fid[u]) - 1];
#pragma unroll
    for (int u = 0; u < MB; ++u) {
      if (f0 + u < nM) {
        const float sgn = fid[u] > 0 ? 1.f : -1.f;
        const float x[4] = {sgn * fl[u].x, sgn * fl[u].y, sgn * fl[u].z, sgn * fl[u].w};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const DF t = df_two_sum(hi[q], x[q]);
          hi[q] = t.hi;
          lo[q] = __fadd_rn(lo[q], t.lo);
        }
      }
    }
  }
  __syncthreads();  // the block's step size (thread 0)
  if (!live || !*s_go) return;
  if (a.res_dbg) a.res_dbg[c] = V4<double>{(double)hi[0] + lo[0], (double)hi[1] + lo[1], (double)hi[2] + lo[2],
                                          (double)hi[3] + lo[3]};
  const float s3 = -*s_bdt * a.vinvf[c];
  DF4* const U = reinterpret_cast<DF4*>(a.U);
  DF4* const U0 = reinterpret_cast<DF4*>(a.U0);
  const DF4 o = U0[c];
  DF base[4] = {{o.hi.x, o.lo.x}, {o.hi.y, o.lo.y}, {o.hi.z, o.lo.z}, {o.hi.w, o.lo.w}};
  if (!k.first) {  // stages 2, 3: beta1 Un + beta2 U (stage 1 is Un + increment, U not read)
    const DF4 u = U[c];
    const DF b1{k.b1h, k.b1l}, b2{k.b2h, k.b2l};
    const DF uu[4] = {{u.hi.x, u.lo.x}, {u.hi.y, u.lo.y}, {u.hi.z, u.lo.z}, {u.hi.w, u.lo.w}};
#pragma unroll
    for (int q = 0; q < 4; ++q) base[q] = df_add(df_mul(b1, base[q]), df_mul(b2, uu[q]));
  }
  DF un[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) un[q] = df_add(base[q], __fmul_rn(s3, __fadd_rn(hi[q], lo[q])));
  const DF4 st{{un[0].hi, un[1].hi, un[2].hi, un[3].hi}, {un[0].lo, un[1].lo, un[2].lo, un[3].lo}};
  U[c] = st;
  if (k.last) U0[c] = st;
  float irf = __fdividef(1.f, un[0].hi);  // 1/rho: fast reciprocal + one Newton step (~1 ulp)
  irf = __fmaf_rn(irf, __fmaf_rn(-un[0].hi, irf, 1.f), irf);
  const DF ke2 = df_div(df_add(df_sqr(un[1]), df_sqr(un[2])), un[0], irf);  // |rhoU|^2 / rho
  const DF e = df_add(un[3], DF{-0.5f * ke2.hi, -0.5f * ke2.lo});
  const float pf = a.gm1f * __fadd_rn(e.hi, e.lo);
  const V4<float> wn{pf, un[1].hi * irf, un[2].hi * irf, pf * irf * a.invRf};
  reinterpret_cast<V4<float>*>(a.W)[c] = wn;
  for (int fi = 0; fi < nM; ++fi) {
    const int f = abs(a.cf[fi * ldc + c]) - 1;
    if (f < a.Nf) continue;
    const int b = f - a.Nf;
    if (a.btype[b] == AFAR_BC_FIXED_INITIAL) continue;  // the ghost keeps its uploaded state
    const V4<double> g = boundary_value(a.btype[b], V4<double>{(double)wn.x, (double)wn.y, (double)wn.z, (double)wn.w},
                                        a.bn[b]);
    reinterpret_cast<V4<float>*>(a.W)[a.Nc + b] = V4<float>{(float)g.x, (float)g.y, (float)g.z, (float)g.w};
  }
}

// evaluateResidual + updateFieldData + updateBoundaryFieldData (+ storeConservedFieldData on the
// last stage), reference cudaFieldOperation.h:183-268, cudaEulerBCs.h:64-95: signed gather of the
// face fluxes in the cell's face order (no atomics), SSP-RK3 combine, conserved -> primitive, and
// the ghost state of this cell's boundary faces from the new state.
template <class P>
__device__ __forceinline__ void update_body(const StageArgs<P>& a, const int blk, const StageCoef& k) {
  // Block constants, computed once by thread 0 (a block never spans two solves): the step size,
  // whether the step is live, and for mixed beta3*dt as a float.  Per-thread code then makes no
  // FP64 operation in the mixed policy (on GB300 even an FP64 comparison costs FP64-pipe time).
  __shared__ double s_dt;
  __shared__ int s_go;
  __shared__ float s_bdt;
  if (threadIdx.x == 0) {
    s_dt = step_dt(a.ctl);
    s_go = s_dt > 0.0;  // past t_end: the step is a no-op
    if constexpr (P::id == PolicyMixed::id) s_bdt = (float)(k.b3 * s_dt);
  }
  const int c = blk * blockDim.x + threadIdx.x;
  if constexpr (P::id == PolicyMixed::id) {
    update_mixed(a, c, k, &s_go, &s_bdt);  // synchronises the block after its flux gather
    return;
  }
  __syncthreads();
  if (c >= a.Nc || !s_go) return;
  const double beta1 = k.b1, beta2 = k.b2, beta3 = k.b3;
  const int last_stage = k.last;
  const double deltaT = s_dt;
  const int ldc = a.ldc;
  const int nM = a.nM[c];
  double Rrho = 0.0, RrhoUx = 0.0, RrhoUy = 0.0, RrhoE = 0.0;
  constexpr int MB = 4;  // face ids, then fluxes, four loads in flight; sums keep the face order
  for (int f0 = 0; f0 < nM; f0 += MB) {
    int fid[MB];
#pragma unroll
    for (int u = 0; u < MB; ++u) fid[u] = (f0 + u < nM) ? a.cf[(f0 + u) * ldc + c] : 1;
    V4<typename P::F> fl[MB];
#pragma unroll
    for (int u = 0; u < MB; ++u) fl[u] = a.flux[abs(fid[u]) - 1];
#pragma unroll
    for (int u = 0; u < MB; ++u) {
      if (f0 + u < nM) {
        const int direction = (fid[u] > 0) - (fid[u] < 0);
        Rrho += direction * (double)fl[u].x;
        RrhoUx += direction * (double)fl[u].y;
        RrhoUy += direction * (double)fl[u].z;
        RrhoE += direction * (double)fl[u].w;
      }
    }
  }
  if (a.res_dbg) a.res_dbg[c] = V4<double>{Rrho, RrhoUx, RrhoUy, RrhoE};
  const V4<double> o = a.U0[c];
  const V4<double> u = a.U[c];
  const double R = a.R;
  const double gamma = a.gamma;  // R/Cv + 1, computed once on the host like GPUevolve.cu:222
  using WT = typename P::W;
  V4<double> un;
  V4<WT> wn;
  if constexpr (P::exact_blend) {  // the reference's eight divisions (cudaFieldOperation.h:229-242)
    const double V = a.vol[c];
    const double rho = beta1 * o.x + beta2 * u.x + beta3 * deltaT * (-Rrho / V);
    const double rhoUx = beta1 * o.y + beta2 * u.y + beta3 * deltaT * (-RrhoUx / V);
    const double rhoUy = beta1 * o.z + beta2 * u.z + beta3 * deltaT * (-RrhoUy / V);
    const double rhoE = beta1 * o.w + beta2 * u.w + beta3 * deltaT * (-RrhoE / V);
    un = V4<double>{rho, rhoUx, rhoUy, rhoE};
    const double p = (gamma - 1.0) * (rhoE - 0.5 * (rhoUx * rhoUx + rhoUy * rhoUy) / rho);
    wn = V4<WT>{(WT)p, (WT)(rhoUx / rho), (WT)(rhoUy / rho), (WT)(p / (R * rho))};
  } else {  // FP64 is scarce on GB300: 1/V precomputed, one division for 1/rho
    const double s3 = -beta3 * deltaT * a.vinv[c];
    const double rho = beta1 * o.x + beta2 * u.x + s3 * Rrho;
    const double rhoUx = beta1 * o.y + beta2 * u.y + s3 * RrhoUx;
    const double rhoUy = beta1 * o.z + beta2 * u.z + s3 * RrhoUy;
    const double rhoE = beta1 * o.w + beta2 * u.w + s3 * RrhoE;
    un = V4<double>{rho, rhoUx, rhoUy, rhoE};
    const double ir = 1.0 / rho;
    const double ux = rhoUx * ir, uy = rhoUy * ir;
    const double p = (gamma - 1.0) * (rhoE - 0.5 * (rhoUx * ux + rhoUy * uy));
    wn = V4<WT>{(WT)p, (WT)ux, (WT)uy, (WT)(p * ir * a.invR)};
  }
  a.U[c] = un;
  if (last_stage) a.U0[c] = un;
  a.W[c] = wn;
  for (int fi = 0; fi < nM; ++fi) {
    const int f = abs(a.cf[fi * ldc + c]) - 1;
    if (f < a.Nf) continue;
    const int b = f - a.Nf;
    if (a.btype[b] == AFAR_BC_FIXED_INITIAL) continue;  // the ghost keeps its uploaded state
    const V4<double> g =
        boundary_value(a.btype[b], V4<double>{(double)wn.x, (double)wn.y, (double)wn.z, (double)wn.w}, a.bn[b]);
    a.W[a.Nc + b] = V4<WT>{(WT)g.x, (WT)g.y, (WT)g.z, (WT)g.w};
  }
}

// ------------------------------------------------------------------------- single-solve kernels
// One solve per launch, arguments by value (read from the parameter bank).
template <class P>
__global__ void __launch_bounds__(128, 5) k_reconstruct_reg(StageArgs<P> a) {
  recon_reg_body<P>(a, blockIdx.x);
}
template <class P, int NF>
__global__ void __launch_bounds__(kTile, 4) k_reconstruct_tile(StageArgs<P> a) {
  extern __shared__ __align__(128) unsigned char sm[];
  recon_tile_body<P, NF>(a, blockIdx.x, sm);
}
template <class P>
__global__ void __launch_bounds__(128) k_reconstruct_staged(StageArgs<P> a) {
  recon_staged_body<P>(a, blockIdx.x);
}
// fp64: its compact staging leaves room for 4 blocks an SM, which 128 registers a thread allow
template <>
__global__ void __launch_bounds__(128, 4) k_reconstruct_staged<PolicyFP64>(StageArgs<PolicyFP64> a) {
  recon_staged_body<PolicyFP64>(a, blockIdx.x);
}
template <class P>
__global__ void __launch_bounds__(128) k_bvd(StageArgs<P> a) {
  bvd_body<P>(a, blockIdx.x);
}
template <class P, bool DT>
__global__ void __launch_bounds__(256) k_flux(StageArgs<P> a) {
  flux_body<P, DT>(a, blockIdx.x);
}
// mixed: 48 registers, 5 blocks an SM (the stage-1 form takes 54 unbounded, and 4 blocks).  The
// bound is for this policy only: a minimum-blocks bound of 1 on the FP64 policies lets ptxas take
// up to 162 registers (one block an SM) where the plain bound keeps 80-120.
template <>
__global__ void __launch_bounds__(256, 5) k_flux<PolicyMixed, false>(StageArgs<PolicyMixed> a) {
  flux_body<PolicyMixed, false>(a, blockIdx.x);
}
template <>
__global__ void __launch_bounds__(256, 5) k_flux<PolicyMixed, true>(StageArgs<PolicyMixed> a) {
  flux_body<PolicyMixed, true>(a, blockIdx.x);
}
template <class P>
__global__ void __launch_bounds__(128) k_update(StageArgs<P> a, const StageCoef k) {
  update_body<P>(a, blockIdx.x, k);
}

// ---------------------------------------------------------------- the multi-point face flux
// An option of the fp64 and mixed policies (no counterpart in the reference, whose flux uses the
// face centre): the face flux as the weighted sum of the fluxes at the face's Gauss points.  The
// switch decisions (troubled cells, BVD) stay those of the face-centre values; at each point the
// state is the O3 value there, or the TVD state extrapolated there with the cell's limited
// gradient, as the cell's switch asks.

// The face values of a cell's side of each internal face at the Gauss points, with the selection
// rules of the face-centre values (recon_*_body): the O3 value where the variable varies over the
// compact stencil by at least 1e-5, else its unlimited linear value; every variable linear in a
// cell of flat temperature.  Runs after the reconstruct, whose gradient it reads.
template <class P>
__global__ void __launch_bounds__(128) k_reconstruct_gauss(StageArgs<P> a) {
  using S = typename P::S;
  using G = typename P::G;
  using WT = typename P::W;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= a.Nc) return;
  const int ldc = a.ldc, nS = a.nS[c], nM = a.nM[c], ng = a.ng, wrow = a.maxS + 1;
  const V4<WT> wc = a.W[c];
  const S pc = (S)wc.x, uxc = (S)wc.y, uyc = (S)wc.z, tc = (S)wc.w;
  S pMax = pc, pMin = pc, uxMax = uxc, uxMin = uxc, uyMax = uyc, uyMin = uyc, tMax = tc, tMin = tc;
  for (int i = 0; i < nM; ++i) {
    const V4<WT> v = a.W[a.sten[i * ldc + c]];
    pMax = fmx((S)v.x, pMax);
    pMin = fmn((S)v.x, pMin);
    uxMax = fmx((S)v.y, uxMax);
    uxMin = fmn((S)v.y, uxMin);
    uyMax = fmx((S)v.z, uyMax);
    uyMin = fmn((S)v.z, uyMin);
    tMax = fmx((S)v.w, tMax);
    tMin = fmn((S)v.w, tMin);
  }
  const V4<G> g0 = a.grad[2 * c], g1 = a.grad[2 * c + 1];  // (px py uxx uxy), (uyx uyy tx ty)
  const S SMALL = AFAR_LIT(S, 1e-5), VSMALL = AFAR_LIT(S, 1e-10);
  const bool flat = fab(tMax - tMin) < VSMALL;
  const bool o3p = !flat && fab(pMax - pMin) >= SMALL, o3ux = !flat && fab(uxMax - uxMin) >= SMALL;
  const bool o3uy = !flat && fab(uyMax - uyMin) >= SMALL, o3t = !flat && fab(tMax - tMin) >= SMALL;
  for (int fi = 0; fi < nM; ++fi) {
    const int fid = a.cf[fi * ldc + c];
    const int f = abs(fid) - 1;
    if (f >= a.Nf) continue;
    const int side = fid < 0;
    for (int k = 0; k < ng; ++k) {
      const V2<G> d = a.sgk[(fi * ng + k) * ldc + c];
      V4<G> o;
      o.x = (G)pc + g0.x * d.x + g0.y * d.y;
      o.y = (G)uxc + g0.z * d.x + g1.x * d.y;
      o.z = (G)uyc + g0.w * d.x + g1.y * d.y;
      o.w = (G)tc + g1.z * d.x + g1.w * d.y;
      if (o3p || o3ux || o3uy || o3t) {
        const S* w = a.wg + (size_t)((fi * ng + k) * wrow) * ldc + c;
        G sp, sux, suy, st;
        if constexpr (std::is_same<G, float>::value) {  // mixed: the difference form of recon_tile_body
          sp = sux = suy = st = G(0);
          for (int j = 0; j < nS; ++j) {
            const S wj = w[(size_t)(j + 1) * ldc];
            const V4<WT> v = a.W[a.sten[j * ldc + c]];
            sp += wj * ((S)v.x - pc);
            sux += wj * ((S)v.y - uxc);
            suy += wj * ((S)v.z - uyc);
            st += wj * ((S)v.w - tc);
          }
          sp += (G)pc;
          sux += (G)uxc;
          suy += (G)uyc;
          st += (G)tc;
        } else {  // fp64: the plain sum, the cell itself first
          const S w0 = w[0];
          sp = w0 * pc;
          sux = w0 * uxc;
          suy = w0 * uyc;
          st = w0 * tc;
          for (int j = 0; j < nS; ++j) {
            const S wj = w[(size_t)(j + 1) * ldc];
            const V4<WT> v = a.W[a.sten[j * ldc + c]];
            sp += wj * (S)v.x;
            sux += wj * (S)v.y;
            suy += wj * (S)v.z;
            st += wj * (S)v.w;
          }
        }
        if (o3p) o.x = sp;
        if (o3ux) o.y = sux;
        if (o3uy) o.z = suy;
        if (o3t) o.w = st;
      }
      a.fvg[(2 * f + side) * ng + k] = o;
    }
  }
}

// The multi-point face flux: for each internal face, the flux at every Gauss point (state
// selection, minimised jumps, central flux and Roe/KFVS dissipation as in flux_body) times the
// point's weight, summed; boundary faces as flux_body (the ghost state is constant along the face,
// so its flux is the same at every point).  The Courant step of the first stage runs as k_delta_t.
template <class P>
__global__ void __launch_bounds__(256) k_flux_gauss(StageArgs<P> a) {
  using S = typename P::S;
  using G = typename P::G;
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  G R, Cv, iR;
  if constexpr (std::is_same<G, float>::value) {
    R = a.Rf;
    Cv = a.Cvf;
    iR = a.invRf;
  } else {
    R = (G)a.R;
    Cv = (G)a.Cv;
    iR = (G)a.invR;
  }
  if (id < a.Nf) {
    const int2 on = a.on[id];
    const int cell[2] = {on.x, on.y};
    const V4<G> fd = a.fd[id];
    const int8_t sw[2] = {a.si[2 * on.x + 1], a.si[2 * on.y + 1]};
    const bool isShock = sw[0] < 0 || sw[1] < 0;
    const V4<G> fs = a.fs[id];
    const G Sfx = fs.x, Sfy = fs.y, magSf = fs.z, nfx = Sfx * fs.w, nfy = Sfy * fs.w;
    const G gam = std::is_same<G, float>::value ? (G)(a.gm1f + 1.f) : (G)a.gamma;
    const G K = G(2) * Cv * iR - G(2);
    G acc[4] = {G(0), G(0), G(0), G(0)};
    for (int k = 0; k < a.ng; ++k) {
      const V2<G> off = a.fgk[id * a.ng + k];
      G st[2][4], T[2][4], rho[2], rhoT[2];
#pragma unroll
      for (int sd = 0; sd < 2; ++sd) {
        const int c = cell[sd];
        const G dx = (sd ? fd.z : fd.x) + off.x, dy = (sd ? fd.w : fd.y) + off.y;
        const V4<typename P::W> w = a.W[c];
        const V4<G> g0 = a.grad[2 * c], g1 = a.grad[2 * c + 1];
        const V4<S> l = a.lim[c];
        T[sd][0] = (G)w.x + l.x * (g0.x * dx + g0.y * dy);
        T[sd][1] = (G)w.y + l.y * (g0.z * dx + g1.x * dy);
        T[sd][2] = (G)w.z + l.z * (g0.w * dx + g1.y * dy);
        T[sd][3] = (G)w.w + l.w * (g1.z * dx + g1.w * dy);
        const V4<G> o3 = a.fvg[(2 * id + sd) * a.ng + k];
        const bool tvd = sw[sd] != 0;
        st[sd][0] = tvd ? T[sd][0] : o3.x;
        st[sd][1] = tvd ? T[sd][1] : o3.y;
        st[sd][2] = tvd ? T[sd][2] : o3.z;
        st[sd][3] = tvd ? T[sd][3] : o3.w;
        rho[sd] = fdiv(st[sd][0] * iR, st[sd][3]);
        rhoT[sd] = fdiv(T[sd][0] * iR, T[sd][3]);
      }
      const G dP = min_delta<G, G>(st[0][0], st[1][0], T[0][0], T[1][0]);
      const G dRho = min_delta<G, G>(rho[0], rho[1], rhoT[0], rhoT[1]);
      const G h = G(0.5);
      G F0 = h * rho[0] * (st[0][1] * Sfx + st[0][2] * Sfy) + h * rho[1] * (st[1][1] * Sfx + st[1][2] * Sfy);
      G F1 = h * (F0 * st[0][1] + st[0][0] * Sfx) + h * (F0 * st[1][1] + st[1][0] * Sfx);
      G F2 = h * (F0 * st[0][2] + st[0][0] * Sfy) + h * (F0 * st[1][2] + st[1][0] * Sfy);
      G F3 = h * F0 * (Cv * st[0][3] + h * (st[0][1] * st[0][1] + st[0][2] * st[0][2]) + R * st[0][3]) +
             h * F0 * (Cv * st[1][3] + h * (st[1][1] * st[1][1] + st[1][2] * st[1][2]) + R * st[1][3]);
      if (isShock)
        kfvs_flux_fast<G>(F0, F1, F2, F3, rho[0], rho[1], st[0][0], st[1][0], st[0][1], st[1][1], st[0][2], st[1][2],
                          st[0][3], st[1][3], R, Cv, K, magSf, nfx, nfy);
      else
        roe_flux_fast<G>(F0, F1, F2, F3, rho[0], rho[1], st[0][1], st[1][1], st[0][2], st[1][2], st[0][3], st[1][3],
                         dP, dRho, R, Cv, gam, magSf, nfx, nfy);
      const G wk = a.gw[k];
      acc[0] += wk * F0;
      acc[1] += wk * F1;
      acc[2] += wk * F2;
      acc[3] += wk * F3;
    }
    a.flux[id] = V4<typename P::F>{(typename P::F)acc[0], (typename P::F)acc[1], (typename P::F)acc[2],
                                   (typename P::F)acc[3]};
  } else if (id < a.Nf + a.Nb) {  // boundary faces: the Euler flux of the ghost state
    const int b = id - a.Nf;
    const V4<typename P::W> wb = a.W[a.Nc + b];
    const V4<G> fs = a.fs[id];
    const G Sfx = fs.x, Sfy = fs.y;
    const G bp = wb.x, bUx = wb.y, bUy = wb.z, bT = wb.w;
    const G rho = bp / (R * bT);
    const G rhoFlux = rho * (bUx * Sfx + bUy * Sfy);
    a.flux[id] = V4<typename P::F>{(typename P::F)rhoFlux, (typename P::F)(rhoFlux * bUx + bp * Sfx),
                                   (typename P::F)(rhoFlux * bUy + bp * Sfy),
                                   (typename P::F)(rhoFlux * (Cv * bT + G(0.5) * (bUx * bUx + bUy * bUy) + bp / rho))};
  }
}

// ------------------------------------------------------------------------- batch kernels
// Many independent solves in one launch: block b works on solve map[b].x (its arguments are
// tab[map[b].x]), as that solve's block map[b].y.  A block never spans two solves, so block-level
// reductions (the CFL minimum, the step size) stay within one solve, and a solve's result does not
// depend on which other solves share the batch.
//
// A block first copies its member's arguments from the table into shared memory (one coalesced
// read of the entry), so the body reads every pointer and constant at shared-memory latency instead
// of one dependent load through L1 per field (the single-solve kernels have them in the parameter
// bank).  Every thread of the block takes part: call it before any thread can leave.
template <class P>
__device__ __forceinline__ const StageArgs<P>& member_args(const StageArgs<P>* __restrict__ tab, const int i) {
  static_assert(sizeof(StageArgs<P>) % 4 == 0, "the argument block is copied as 32-bit words");
  __shared__ __align__(16) unsigned raw[sizeof(StageArgs<P>) / 4];
  const unsigned* src = reinterpret_cast<const unsigned*>(tab + i);
  for (int w = threadIdx.x; w < (int)(sizeof(StageArgs<P>) / 4); w += blockDim.x) raw[w] = __ldg(src + w);
  __syncthreads();
  return *reinterpret_cast<const StageArgs<P>*>(raw);
}
template <class P, int NF>
__global__ void __launch_bounds__(kTile, 4) kb_reconstruct_tile(const StageArgs<P>* __restrict__ tab,
                                                                const int2* __restrict__ map) {
  extern __shared__ __align__(128) unsigned char sm[];
  const int2 m = map[blockIdx.x];
  recon_tile_body<P, NF>(member_args(tab, m.x), m.y, sm);
}
template <class P>
__global__ void __launch_bounds__(128) kb_reconstruct_staged(const StageArgs<P>* __restrict__ tab,
                                                             const int2* __restrict__ map) {
  const int2 m = map[blockIdx.x];
  recon_staged_body<P>(member_args(tab, m.x), m.y);
}
template <>
__global__ void __launch_bounds__(128, 4) kb_reconstruct_staged<PolicyFP64>(const StageArgs<PolicyFP64>* __restrict__ tab,
                                                                            const int2* __restrict__ map) {
  const int2 m = map[blockIdx.x];
  recon_staged_body<PolicyFP64>(member_args(tab, m.x), m.y);
}
// the register-pass reconstruct of the mixed policy over the members the autotuner gave it
template <class P>
__global__ void __launch_bounds__(128, 5) kb_reconstruct_reg(const StageArgs<P>* __restrict__ tab,
                                                            const int2* __restrict__ map) {
  const int2 m = map[blockIdx.x];
  recon_reg_body<P>(member_args(tab, m.x), m.y);
}
// BVD and flux in blocks of B threads (the batch autotuner's choice; the map's blocks are B cells
// or faces of one member).  mixed BVD: 32 registers, the full 64 warps per SM; fp64: 40 warps.
template <class P, int B>
__global__ void __launch_bounds__(B, (P::id == PolicyMixed::id ? 2048 : 1280) / B) kb_bvd(
    const StageArgs<P>* __restrict__ tab, const int2* __restrict__ map) {
  const int2 m = map[blockIdx.x];
  bvd_body<P>(tab[m.x], m.y);  // staging its arguments cost more than it saved (32 registers)
}
template <class P, bool DT, int B>
__global__ void __launch_bounds__(B) kb_flux(const StageArgs<P>* __restrict__ tab, const int2* __restrict__ map) {
  const int2 m = map[blockIdx.x];
  flux_body<P, DT>(member_args(tab, m.x), m.y);
}
template <class P>
__global__ void __launch_bounds__(128) kb_update(const StageArgs<P>* __restrict__ tab, const int2* __restrict__ map,
                                                 const StageCoef k) {
  const int2 m = map[blockIdx.x];
  update_body<P>(member_args(tab, m.x), m.y, k);
}

// Closes a step: advance time, record the step, re-arm the CFL minimum for the next step.
__device__ __forceinline__ void finish_one(StepCtl* ctl) {
  const double dt = step_dt(ctl);
  if (dt > 0.0) {
    ctl->t += dt;
    ctl->steps += 1;
    ctl->last_dt = dt;
    if (ctl->write_interval > 0.0)  // passed a write time (within rounding): aim at the next one
      for (int k = 0; k < 4 && ctl->t >= (double)(ctl->write_index + 1) * ctl->write_interval * (1.0 - 1e-12); ++k)
        ctl->write_index += 1;
  }
  ctl->dt_bits = (unsigned long long)__double_as_longlong(1e5);
}
template <class P>
__global__ void kb_finish_step(const StageArgs<P>* __restrict__ tab, const int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) finish_one(tab[i].ctl);
}

__global__ void k_finish_step(StepCtl* ctl) {
  if (threadIdx.x == 0 && blockIdx.x == 0) finish_one(ctl);
}

// The CFL step alone (adjustTimeStep of the drop-in API): min over internal faces into *bits.
// With ctl != nullptr (the step graph) it reduces into ctl->dt_bits with ctl->cfl, and does nothing
// when the step size is fixed.
template <class P>
__global__ void __launch_bounds__(256) k_delta_t(StageArgs<P> a, double CFL, unsigned long long* bits,
                                                 const StepCtl* ctl) {
  if (ctl) {
    if (ctl->dt_fixed > 0.0) return;
    CFL = ctl->cfl;
  }
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  double dtf = 1e5;
  if (id < a.Nf) {
    const int2 on = a.on[id];
    const V4<typename P::W> Wo = a.W[on.x], Wn = a.W[on.y];
    const V4<typename P::G> fs = a.fs[id];
    const double sfx = (double)fs.x, sfy = (double)fs.y, msf = (double)fs.z;
    const V2<double> g = a.dtg[id];
    const double deltaR = g.x, fraction = g.y, Rd = a.R, Cvd = a.Cv;
    dtf = CFL * deltaR * msf /
          ((1.0 - fraction) * fabs((double)Wo.y * sfx + (double)Wo.z * sfy) +
           fraction * fabs((double)Wn.y * sfx + (double)Wn.z * sfy) +
           sqrt((Rd / Cvd + 1.0) * Rd * ((1.0 - fraction) * (double)Wo.w + fraction * (double)Wn.w)) * msf);
  }
  unsigned long long v = (unsigned long long)__double_as_longlong(dtf);
  if (!(dtf >= 0.0)) v = 0x7FF0000000000000ull;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long u = __shfl_xor_sync(0xffffffffu, v, o);
    v = u < v ? u : v;
  }
  if ((threadIdx.x & 31) == 0) atomicMin(bits, v);
}

// The Courant step of the mixed policy for afar_adjustTimeStep: the FP32 estimate of its fused
// stage-1 flux (same expression), warp minimum on the float bits, one atomicMin per warp on the
// double's bits.  No FP64 arithmetic per face.
__global__ void __launch_bounds__(256) k_delta_t_mixed(StageArgs<PolicyMixed> a, const float cfl,
                                                       unsigned long long* bits) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  float dtf = 1e5f;
  if (id < a.Nf) {
    const int2 on = a.on[id];
    const V4<float> Wo = a.W[on.x], Wn = a.W[on.y];
    const V4<float> fs = a.fs[id];
    const float Sfx = fs.x, Sfy = fs.y, magSf = fs.z;
    const V2<float> g = a.dtgf[id];
    dtf = courant_dt_f32(cfl, g.x, magSf, courant_den_f32(g.y, magSf, Sfx, Sfy, Wo, Wn, a.gRf));
  }
  unsigned v = (unsigned)__float_as_int(dtf);
  if (!(dtf >= 0.f)) v = 0x7F800000u;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned u = __shfl_xor_sync(0xffffffffu, v, o);
    v = u < v ? u : v;
  }
  if ((threadIdx.x & 31) == 0) {
    const unsigned long long b = v >= 0x7F800000u
                                     ? 0x7FF0000000000000ull
                                     : (unsigned long long)__double_as_longlong((double)__int_as_float((int)v));
    atomicMin(bits, b);
  }
}

// ---------------------------------------------------------------------------------- setup kernels

// A coordinate difference taken to the nearest periodic image (L > 0), else unchanged.
__device__ __forceinline__ double wrapd(const double d, const double L) { return L > 0.0 ? d - L * rint(d / L) : d; }

// calcLeastSquareMatrix (reference cudaFieldOperation.h:91-120) into the slot-major matrix, in
// FP64 math, stored in the policy's operator type.
template <class P>
__global__ void k_setup_lsm(StageArgs<P> a, V2<typename P::S>* lsm, float* lsm_ref_layout, int maxM_ref) {
  using S = typename P::S;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= a.Nc) return;
  const int m = a.nM[c];
  double Sxx = 0.0, Sxy = 0.0, Syy = 0.0;
  const double x0 = a.cellC[c].x, y0 = a.cellC[c].y;
  for (int i = 0; i < m; ++i) {
    const int j = a.sten[i * a.ldc + c];
    const double dx = wrapd(a.cellC[j].x - x0, a.px), dy = wrapd(a.cellC[j].y - y0, a.py);
    Sxx += dx * dx;
    Sxy += dx * dy;
    Syy += dy * dy;
  }
  for (int i = 0; i < m; ++i) {
    const int j = a.sten[i * a.ldc + c];
    const double dx = wrapd(a.cellC[j].x - x0, a.px), dy = wrapd(a.cellC[j].y - y0, a.py);
    const S m1 = (Syy * dx - Sxy * dy) / (Sxx * Syy - Sxy * Sxy);
    const S m2 = (-Sxy * dx + Sxx * dy) / (Sxx * Syy - Sxy * Sxy);
    lsm[i * a.ldc + c] = V2<S>{m1, m2};
    if (lsm_ref_layout) {
      lsm_ref_layout[2 * (size_t)maxM_ref * c + 2 * i] = (float)m1;
      lsm_ref_layout[2 * (size_t)maxM_ref * c + 2 * i + 1] = (float)m2;
    }
  }
}

// Geometry constants of each (cell, face slot): the face offset from the cell centre and the
// (delta r, fraction) pair reconstruct uses, with the reference's expressions
// (cudaLimiter.h:258-262), so the values are bit-identical to what its kernel computes per stage.
template <class P>
__global__ void k_setup_slot_geom(StageArgs<P> a, const V4<double>* faceXY) {
  using S = typename P::S;
  using G = typename P::G;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= a.Nc) return;
  const int m = a.nM[c];
  const double x0 = a.cellC[c].x, y0 = a.cellC[c].y;
  V2<G>* sg = const_cast<V2<G>*>(a.sg);
  V2<S>* sr = const_cast<V2<S>*>(a.sr);
  for (int fi = 0; fi < m; ++fi) {
    const int f = abs(a.cf[fi * a.ldc + c]) - 1;
    const double dx = wrapd(faceXY[f].x - x0, a.px);
    const double dy = wrapd(faceXY[f].y - y0, a.py);
    sg[fi * a.ldc + c] = V2<G>{(G)dx, (G)dy};
    S dR = S(1), fr = S(0);
    if (f < a.Nf) {
      const int nb = a.sten[fi * a.ldc + c];
      const double nx = wrapd(a.cellC[nb].x - x0, a.px), ny = wrapd(a.cellC[nb].y - y0, a.py);
      const float deltaR = hypot(nx, ny);
      const float fraction = sqrt(dx * dx + dy * dy) / deltaR;
      if (P::id == PolicyFP64::id) {
        const double dRd = hypot(nx, ny);
        dR = (S)dRd;
        fr = (S)(sqrt(dx * dx + dy * dy) / dRd);
      } else {
        dR = (S)deltaR;
        fr = (S)fraction;
      }
    }
    sr[fi * a.ldc + c] = V2<S>{dR, fr};
  }
}

// Per-face constants: offsets of the face centre from owner and neighbour (evaluateFlux :178-182),
// the CFL geometry (setDeltaT :145-146), face vectors, boundary unit normals (symmetryBoundary.h).
template <class P>
__global__ void k_setup_face_geom(StageArgs<P> a, const V4<double>* faceXY, const V4<double>* faceS) {
  using G = typename P::G;
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= a.Nf + a.Nb) return;
  const V4<double> xy = faceXY[f];  // x, y
  const V4<double> s = faceS[f];    // Sfx, Sfy, magSf
  // fs.w: 1/|Sf| for the dissipation of the policies without bit parity (the ref policy's flux
  // divides like the reference)
  const_cast<V4<G>*>(a.fs)[f] = V4<G>{(G)s.x, (G)s.y, (G)s.z, P::id == PolicyRef::id ? G(0) : (G)(1.0 / s.z)};
  if (f < a.Nf) {
    const int2 on = a.on[f];
    const V2<double> co = a.cellC[on.x], cn = a.cellC[on.y];
    const double oxd = wrapd(xy.x - co.x, a.px), oyd = wrapd(xy.y - co.y, a.py);
    const double nxd = wrapd(xy.x - cn.x, a.px), nyd = wrapd(xy.y - cn.y, a.py);
    const_cast<V4<G>*>(a.fd)[f] = V4<G>{(G)oxd, (G)oyd, (G)nxd, (G)nyd};
    const double deltaR = hypot(wrapd(cn.x - co.x, a.px), wrapd(cn.y - co.y, a.py));
    const double fraction = hypot(oxd, oyd) / deltaR;
    const_cast<V2<double>*>(a.dtg)[f] = V2<double>{deltaR, fraction};
  } else {
    const int b = f - a.Nf;
    const_cast<V2<double>*>(a.bn)[b] = V2<double>{s.x / s.z, s.y / s.z};
  }
}

// The multi-point face flux's per-cell arrays from the face-ordered inputs: each cell slot's O3
// weights at the points (its side's row of rbfg [face][side][point][maxS+1]; zeros past the stencil
// and for boundary faces) and the points minus the cell centre (nearest periodic image).
template <class P>
__global__ void k_setup_gauss(StageArgs<P> a, const double* rbfg, const double* pts) {
  using S = typename P::S;
  using G = typename P::G;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= a.Nc) return;
  const int ng = a.ng, nmax = a.maxS + 1, ldc = a.ldc;
  S* wg = const_cast<S*>(a.wg);
  V2<G>* sgk = const_cast<V2<G>*>(a.sgk);
  const double x0 = a.cellC[c].x, y0 = a.cellC[c].y;
  for (int fi = 0; fi < a.nM[c]; ++fi) {
    const int fid = a.cf[fi * ldc + c];
    const int f = abs(fid) - 1;
    if (f >= a.Nf) continue;
    const int side = fid < 0;
    for (int k = 0; k < ng; ++k) {
      const double px = pts[2 * ((size_t)f * ng + k)], py = pts[2 * ((size_t)f * ng + k) + 1];
      sgk[(fi * ng + k) * ldc + c] = V2<G>{(G)wrapd(px - x0, a.px), (G)wrapd(py - y0, a.py)};
      const double* src = rbfg + (((size_t)f * 2 + side) * ng + k) * nmax;
      for (int j = 0; j <= a.nS[c]; ++j) wg[(size_t)((fi * ng + k) * nmax + j) * ldc + c] = (S)src[j];
    }
  }
}
template <class P>
__global__ void k_setup_gauss_faces(StageArgs<P> a, const double* pts, const V4<double>* faceXY) {
  using G = typename P::G;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.Nf * a.ng) return;
  const int f = i / a.ng;
  const V4<double> xy = faceXY[f];
  const_cast<V2<G>*>(a.fgk)[i] = V2<G>{(G)wrapd(pts[2 * (size_t)i] - xy.x, a.px), (G)wrapd(pts[2 * (size_t)i + 1] - xy.y, a.py)};
}

}  // namespace afar
