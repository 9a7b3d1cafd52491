// wacsf_grouped.cuh - FP32 descriptor kernels for grouped angular SF sets
// (included by wacsf.cu inside its anonymous namespace).
//
// Taken when every angular SF shares one cutoff, there are at most 4
// angular alphas and at most 8 combinations of (lambda, integer zeta) - the
// usual wACSF sets, including every synthetic model here.  An angular SF s is
// then the pair (alpha q_s, combination c_s), and for a triplet
//   G_s term = 2^(1-zeta) A_c(cos) E_q F,   A_c = (1 + lambda_c cos)^zeta_c,
//   E_q = exp(-alpha_q (rij^2 + rik^2 + rjk^2)),  F = fc(rij) fc(rik) fc(rjk),
// so per pair only NAL exponentials and NC powers are distinct:
//  - forward: the pair adds A_c E_q F (and its w_j w_k weighted copy) to a
//    NAL x NC register grid; every SF reads its cell at the end;
//  - gradient: dE/dG is contracted first into per-atom NAL x NC matrices
//    UA = sum_s 2^(1-zeta) dE/dG_s, UB = the same for the weighted copies,
//    so the pair's chain-rule scalars need NAL x NC multiply-adds in total.
// Pairs beyond the cutoff are dropped by a per-warp ballot queue before the
// arithmetic, so all lanes work on contributing pairs.  The gradient kernel
// accumulates slot gradients in fixed point by int32 shared-memory atomics
// (exact integer sums, so the same in every run) and scatters the forces
// with FP64 atomics in place of the reverse-slot gather (their order, hence
// the forces' last bits, may vary between runs; the FP64 path keeps the
// deterministic round-robin schedule).

// per-warp ring queues of contributing pairs: the forward kernel screens two
// 32-candidate batches per step (at most 31 + 64 entries pending), the
// gradient kernel's overflow path one batch (at most 31 + 32)
constexpr int kPairQFwd = 128;
constexpr int kPairQBwd = 64;
// resident blocks per SM the grouped kernels are compiled for: the forward
// kernel 6 (80 registers a thread; at 7 and 72 registers it ran 4 % slower),
// the gradient kernel 7 (72 registers) where the instantiation compiles
// without spilling, 6 otherwise.  The launchers ask for the largest
// shared-memory carve-out so that the per-warp slot tables of those blocks
// fit, and size the grid by the occupancy the compiled kernel reaches.
constexpr int kGrpMinBlocks = 6;
template <int NAL, int NC, bool STD>
constexpr int grp_bwd_blocks() {
  return ((NAL <= 2 && (STD || NC <= 2)) || (NAL == 1 && NC <= 4)) ? 7 : 6;
}

// Per-warp shared-memory layout of the grouped kernels: packed slot records
// (a pair reads its two slots with four 128-bit loads; the angular
// exponential exp(-alpha (rij^2 + rik^2 + rjk^2)) is formed per pair from the
// three squared lengths) and the per-cutoff tables of the radial terms.
//   a[q] = (dx, dy, dz, r)        b[q] = (1/r, w, fc, fc') at the angular cutoff
//   fc[g][q], dfc[g][q]           cutoff function of every cutoff group g, kept
//                                 only with several groups (with one, b holds it)
//   rco[s]                        (kx, rs, dE/dG_d, dE/dG_{d+nsf}) of radial SF s
//                                 (gradient kernel)
//   g6[q][c][2]                   slot gradient component c in fixed point,
//                                 g6[q][c][0] 2^-9 + g6[q][c][1] 2^-29
//                                 (gradient kernel): a slot's six words are
//                                 adjacent, so a pair's six atomic adds share
//                                 one address
//   dg[D]                         dE/dG (gradient kernel)
struct GLay {
  float4 *a, *b, *rco;
  float *fc, *dfc, *dg;
  int *g6;
};

__host__ __device__ inline int grp_fc_groups(int nrc) { return nrc > 1 ? nrc : 0; }

__host__ __device__ inline size_t grp_warp_floats(int capS, int nrc, int D, int nrad, bool fwd) {
  const size_t n = (size_t)8 * capS + (size_t)grp_fc_groups(nrc) * capS * (fwd ? 1 : 2) +
                   (fwd ? 0 : (size_t)4 * nrad + (size_t)6 * capS + D);
  return (n + 3) / 4 * 4;  // keeps every warp's records 16-byte aligned
}

__device__ __forceinline__ GLay grp_carve(unsigned char *raw, int warp, int capS, int nrc, int D,
                                          int nrad, bool fwd) {
  float *base = reinterpret_cast<float *>(raw + kTableBytes(sizeof(SFT<float>))) +
                grp_warp_floats(capS, nrc, D, nrad, fwd) * warp;
  GLay L;
  L.a = reinterpret_cast<float4 *>(base);
  L.b = L.a + capS;
  L.rco = fwd ? nullptr : L.b + capS;  // gradient kernel: per-SF radial records
  // g6 follows the 16-byte records, so every slot's words are 8-byte aligned
  L.g6 = fwd ? nullptr : reinterpret_cast<int *>(L.rco + nrad);
  L.fc = fwd ? reinterpret_cast<float *>(L.b + capS) : reinterpret_cast<float *>(L.g6 + 6 * capS);
  const size_t nfc = (size_t)grp_fc_groups(nrc) * capS;
  L.dfc = fwd ? nullptr : L.fc + nfc;
  L.dg = fwd ? nullptr : L.dfc + nfc;
  return L;
}

// Stages atom i's slots from the FP32 records of the neighbour kernel; the
// forward and gradient kernels stage through this one routine, so they
// differentiate the same function.  The staged functions keep the accurate
// libm forms: with __sincosf / __expf / __fdividef here the tensor-core form's
// force error on a stiff Si model (forces ~150 eV/A) rose from within
// 20 meV/A to 23 meV/A.
__device__ __forceinline__ int grp_stage(const GLay &L, const SFT<float> &sf, int i, int cap,
                                         int capS, int lane, int rci, const int *__restrict__ cnt,
                                         const float4 *__restrict__ d32,
                                         const float *__restrict__ w32, bool want_dfc) {
  const int P = min(cnt[i], capS);
  const int nrc = sf.nrc, nal = sf.nalpha;
  for (int q = lane; q < P; q += 32) {
    const float4 g = d32[(size_t)i * cap + q];
    const float r = g.w, w = w32[(size_t)i * cap + q];
    float fa = 0.f, dfa = 0.f;
    for (int gr = 0; gr < nrc; ++gr) {
      float fcv = 0.f, dfcv = 0.f;
      if (r <= sf.rc_val[gr]) {
        const float x = sf.pi_over_rc[gr] * r;
        if (want_dfc) {
          float sn, cs;
          sincosf(x, &sn, &cs);
          fcv = 0.5f * (cs + 1.f);
          dfcv = -0.5f * sn * sf.pi_over_rc[gr];
        } else {
          fcv = 0.5f * (cosf(x) + 1.f);
        }
      }
      if (nrc > 1) {
        L.fc[(size_t)gr * capS + q] = fcv;
        if (want_dfc) L.dfc[(size_t)gr * capS + q] = dfcv;
      }
      if (gr == rci) {
        fa = fcv;
        dfa = dfcv;
      }
    }
    L.a[q] = g;
    L.b[q] = make_float4(1.f / r, w, fa, dfa);
  }
  return P;
}

__device__ __forceinline__ float f4get(const float4 &v, int t) {
  return t == 0 ? v.x : (t == 1 ? v.y : (t == 2 ? v.z : v.w));
}

// b^iz and b^(iz-1) for integer zeta >= 1 (branch-free up to 4)
__device__ __forceinline__ float pow_iz(float b, int iz, float *pm1) {
  const float b2 = b * b;
  float p;
  if (iz <= 4) {
    p = iz == 1 ? 1.f : (iz == 2 ? b : (iz == 3 ? b2 : b2 * b));
  } else {
    p = b2 * b2;
    for (int t = 5; t < iz; ++t) p *= b;
  }
  *pm1 = p;
  return p * b;
}

// (1 + cos), (1 - cos), (1 + cos)^2, (1 - cos)^2, (1 + cos)^4, (1 - cos)^4 in the
// degree-4 Bernstein basis u^n w^(4-n), u = (1 + cos)/2, w = 1 - u:
// 2u = 2u(u+w)^3, 2w = 2w(u+w)^3, 4u^2 = 4u^2(u+w)^2, ..., 16u^4, 16w^4
__constant__ float kBern[6][5] = {{0.f, 2.f, 6.f, 6.f, 2.f},  {2.f, 6.f, 6.f, 2.f, 0.f},
                                  {0.f, 0.f, 4.f, 8.f, 4.f},  {4.f, 8.f, 4.f, 0.f, 0.f},
                                  {0.f, 0.f, 0.f, 0.f, 16.f}, {16.f, 0.f, 0.f, 0.f, 0.f}};

// A_c = (1 + lambda_c cos)^zeta_c and dA_c/dcos for the combinations of a
// pair: closed form for the standard set (STD: c = 2 log2(zeta) + (lambda < 0)),
// integer powers otherwise
template <int NC, bool STD>
__device__ __forceinline__ void ang_powers(float cosv, const float *clam, const int *ciz,
                                           float *A, float *dAl) {
  if constexpr (STD && NC == 6) {
    const float bp = 1.f + cosv, bm = 1.f - cosv;
    const float bp2 = bp * bp, bm2 = bm * bm;
    A[0] = bp;
    A[1] = bm;
    A[2] = bp2;
    A[3] = bm2;
    A[4] = bp2 * bp2;
    A[5] = bm2 * bm2;
    if (dAl) {
      dAl[0] = 1.f;
      dAl[1] = -1.f;
      dAl[2] = 2.f * bp;
      dAl[3] = -2.f * bm;
      dAl[4] = 4.f * bp * bp2;
      dAl[5] = -4.f * bm * bm2;
    }
  } else {
#pragma unroll
    for (int cc = 0; cc < NC; ++cc) {
      float p;  // base^(zeta-1)
      A[cc] = pow_iz(1.f + clam[cc] * cosv, ciz[cc], &p);
      if (dAl) dAl[cc] = (float)ciz[cc] * p * clam[cc];  // d A / d cos
    }
  }
}

// Walks the upper triangle of P slots, screens pairs (r_jk <= rc) and calls
// `work(j, k, rjk^2, valid)` on all 32 lanes for every batch of up to 32
// contributing pairs (valid is false on the idle lanes of the last batch;
// the valid lanes sit below the invalid ones).  Rows r and P - 2 - r are
// walked together (they hold P candidates between them, so a lane finds its
// (j, k) with two comparisons and no loop); the pairs of one row j are
// contiguous in the stream, so equal j values are contiguous in a batch.
template <int Q, typename Work>
__device__ __forceinline__ void pair_stream(const float4 *__restrict__ A, int P, float rc, int lane,
                                            int *qjk, float *qc2, Work work) {
  const float rc2 = rc * rc;
  const unsigned lt = (1u << lane) - 1u;
  int qh = 0, qn = 0;  // ring queue: entries [qh, qn) are pending
  // candidate t of the row pair (r, r2): its (j, k), whether it contributes,
  // and r_jk^2.  Branch-free: a lane past the row pair's end reads slots 0
  // and 1 (P > 1) and reports no pair
  auto cand = [&](int r, int r2, int n1, int tot, int t, int &j, int &k, float &c2) {
    const bool in = t < tot, second = t >= n1;
    j = in ? (second ? r2 : r) : 0;
    k = in ? (second ? r2 + 1 + (t - n1) : r + 1 + t) : 1;
    const float4 aj = A[j], ak = A[k];
    const float cx = aj.x - ak.x, cy = aj.y - ak.y, cz = aj.z - ak.z;
    c2 = cx * cx + cy * cy + cz * cz;
    return in & (aj.w <= rc) & (ak.w <= rc) & (c2 <= rc2);
  };
  // queue the contributing candidates in lane order; every lane stores, the
  // others into their own spare entry past the ring (entries Q + lane)
  auto push = [&](bool valid, int j, int k, float c2) {
    const unsigned m = __ballot_sync(0xffffffffu, valid);
    const int e = valid ? (qn + __popc(m & lt)) & (Q - 1) : Q + lane;
    qjk[e] = j | (k << 16);
    qc2[e] = c2;
    qn += __popc(m);
  };
  const int nfold = P / 2;  // row pairs (r, P - 2 - r); the middle row of an even P is alone
  for (int r = 0; r < nfold; ++r) {
    const int r2 = P - 2 - r;
    const int n1 = P - 1 - r;                // candidates of row r
    const int tot = r2 > r ? P : n1;         // with row r2's r + 1
    // Q / 64 batches of 32 candidates per step (at most 31 + 32 Q / 64 < Q
    // entries pending): their loads and distances are independent, which
    // hides the shared-memory latency of the screen
    constexpr int NB = Q / 64 > 0 ? Q / 64 : 1;
    for (int base = 0; base < tot; base += 32 * NB) {
      int jb[NB], kb[NB];
      float cb[NB];
      bool vb[NB];
#pragma unroll
      for (int b = 0; b < NB; ++b) vb[b] = cand(r, r2, n1, tot, base + 32 * b + lane, jb[b], kb[b], cb[b]);
#pragma unroll
      for (int b = 0; b < NB; ++b) push(vb[b], jb[b], kb[b], cb[b]);
      __syncwarp();
      while (qn - qh >= 32) {
        const int e = (qh + lane) & (Q - 1);
        const int jk = qjk[e];
        const float cc = qc2[e];
        __syncwarp();
        work(jk & 0xffff, jk >> 16, cc, true);
        qh += 32;
      }
    }
  }
  if (qn > qh) {
    const int e = (qh + lane) & (Q - 1);
    const bool have = lane < qn - qh;
    const int jk = have ? qjk[e] : (0 | (1 << 16));
    const float cc = have ? qc2[e] : 1.f;
    __syncwarp();
    work(jk & 0xffff, jk >> 16, cc, have);
  }
  __syncwarp();
}

constexpr float kLog2e = 1.4426950408889634f;
constexpr float kTwoLn2 = 1.3862943611198906f;

// 2^x on the MUFU pipe (the __expf form: exp(y) = ex2(y log2 e))
__device__ __forceinline__ float ex2f(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Slot gradients in fixed point.  A term v is split as
//   v = h 2^-9 + l 2^-29 + e,  |e| <= 2^-30,  |h| <= 2^20,  |l| <= 2^19,
// and h and l are summed by native int32 shared-memory atomic adds (an FP32
// atomic add is a compare-and-swap loop).  Integer sums do not depend on the
// order of the adds, so the slot gradients are the same in every run.  The
// rounding uses the 1.5 2^23 shifter (exact for |x| < 2^22), so the split
// stays on the FP32 and integer pipes.  A slot receives at most 2047 terms
// (one radial write, at most capS - 1 k-side pairs and capS - 1 j-side
// partial sums; capS <= 1024, since the gradient kernel's per-warp tables
// take at least 56 bytes per slot and four warps share the 227 KB of a
// block), so with |v| <= kFxMax both sums fit int32.  A
// term beyond kFxMax, or not finite, marks the atom (`bad`), and the kernel
// raises kFlagForceRange (tested once per vector, as |x| + |y| + |z|).
constexpr float kFxShift = 12582912.f;  // 1.5 2^23
constexpr int kFxShiftBits = 0x4B400000;
constexpr float kFxMax = 2047.f;  // eV/A per term
__device__ __forceinline__ void fx_split(float v, int &h, int &l) {
  const float ts = fmaf(v, 512.f, kFxShift);              // v 2^9 rounded, plus the shifter
  h = __float_as_int(ts) - kFxShiftBits;
  const float hf = ts - kFxShift;                          // exact
  const float u = fmaf(hf, -1048576.f, v * 536870912.f);  // (v 2^9 - hf) 2^20, exact
  l = __float_as_int(u + kFxShift) - kFxShiftBits;
}
__device__ __forceinline__ void slot_add(const GLay &L, int q, float x, float y, float z,
                                         bool &bad) {
  bad |= !(fabsf(x) + fabsf(y) + fabsf(z) <= kFxMax);
  int *w = L.g6 + 6 * q;
  int h, l;
  fx_split(x, h, l);
  atomicAdd(w + 0, h);
  atomicAdd(w + 1, l);
  fx_split(y, h, l);
  atomicAdd(w + 2, h);
  atomicAdd(w + 3, l);
  fx_split(z, h, l);
  atomicAdd(w + 4, h);
  atomicAdd(w + 5, l);
}
__device__ __forceinline__ void slot_set(const GLay &L, int q, float x, float y, float z,
                                         bool &bad) {
  bad |= !(fabsf(x) + fabsf(y) + fabsf(z) <= kFxMax);
  int2 *w = reinterpret_cast<int2 *>(L.g6 + 6 * q);
  int h, l;
  fx_split(x, h, l);
  w[0] = make_int2(h, l);
  fx_split(y, h, l);
  w[1] = make_int2(h, l);
  fx_split(z, h, l);
  w[2] = make_int2(h, l);
}
__device__ __forceinline__ float fx_value(int2 v) {
  return fmaf((float)v.x, 0.001953125f, (float)v.y * 1.86264514923095703125e-09f);
}

// radial part of the forward kernel: one SF per lane over the slots in
// order, exp(-alpha (r - rs)^2) = 2^(kx (r - rs)^2) with kx = -alpha log2 e.
// A term beyond its cutoff has fc = 0 and adds exactly zero.  With a single
// cutoff group the slot's fc and weight come from its packed record.
__device__ __forceinline__ void radial_fwd(const GLay &L, const SFT<float> &sf, int P, int capS,
                                           int lane, float *Gi) {
  for (int s = lane; s < sf.nrad; s += 32) {
    const float kx = -sf.rad_alpha[s] * kLog2e, rs = sf.rad_rs[s];
    float acc = 0.f, accw = 0.f;
    if (sf.nrc == 1) {
#pragma unroll 4
      for (int q = 0; q < P; ++q) {
        const float4 bq = L.b[q];
        const float u = L.a[q].w - rs;
        const float v = ex2f(kx * (u * u)) * bq.z;
        acc += v;
        accw = fmaf(v, bq.y, accw);
      }
    } else {
      const float *f_ = L.fc + sf.rad_rc[s] * capS;
#pragma unroll 4
      for (int q = 0; q < P; ++q) {
        const float u = L.a[q].w - rs;
        const float v = ex2f(kx * (u * u)) * f_[q];
        acc += v;
        accw = fmaf(v, L.b[q].y, accw);
      }
    }
    const int d = sf.rad_d[s];
    Gi[d] = acc;
    Gi[d + sf.nsf] = accw;
  }
}

template <int NAL, int NC, bool STD>
__global__ void __launch_bounds__(32 * kWarpsPerBlock, kGrpMinBlocks)
    k_wacsf_fwd_grp(int N, int cap, int capS, const int *__restrict__ cnt,
                    const double4 *__restrict__ xyzr, const int *__restrict__ nj,
                    const double4 *__restrict__ apos, const float4 *__restrict__ d32,
                    const float *__restrict__ w32, const SFT<float> *__restrict__ sfg,
                    float *__restrict__ G, unsigned short *__restrict__ pairs,
                    int *__restrict__ pcount, int pcap) {
  (void)xyzr;
  (void)nj;
  (void)apos;
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ int s_qjk[kWarpsPerBlock][kPairQFwd + 32];  // ring + the lanes' spare entries
  __shared__ float s_qc2[kWarpsPerBlock][kPairQFwd + 32];
  __shared__ float s_acc[kWarpsPerBlock][2 * NAL * NC];
  __shared__ float s_out[kWarpsPerBlock][(STD && NC == 6) ? 2 * NAL * NC : 1];
  load_table<float>(smraw, sfg);
  const SFT<float> &sf = *reinterpret_cast<const SFT<float> *>(smraw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nal = sf.nalpha, D = sf.D, nsf = sf.nsf, nang = sf.nang;
  const GLay L = grp_carve(smraw, warp, capS, sf.nrc, D, sf.nrad, true);
  const int rci = nang > 0 ? sf.ang_grp_rc[0] : 0;
  const float rc = sf.rc_val[rci], pirc = sf.pi_over_rc[rci];
  float alv[NAL], kal[NAL], clam[NC];
  int ciz[NC];
#pragma unroll
  for (int q = 0; q < NAL; ++q) {
    alv[q] = q < nal ? sf.alpha_val[q] : 0.f;
    kal[q] = -alv[q] * kLog2e;
  }
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    clam[c] = sf.comb_lam[c];
    ciz[c] = sf.comb_iz[c];
  }
  for (int i = blockIdx.x * kWarpsPerBlock + warp; i < N; i += gridDim.x * kWarpsPerBlock) {
    const int P = grp_stage(L, sf, i, cap, capS, lane, rci, cnt, d32, w32, false);
    __syncwarp();
    float *Gi = G + (size_t)i * D;
    radial_fwd(L, sf, P, capS, lane, Gi);
    if (nang == 0) continue;
    // the standard set accumulates the degree-4 Bernstein moments
    // sum EF u^n w^(4-n) (u = (1 + cos)/2, w = 1 - u), from which every
    // (1 +- cos)^zeta follows with non-negative weights (kBern); other sets
    // accumulate their NC powers directly
    constexpr bool kB = STD && NC == 6;
    constexpr int NB = kB ? 5 : NC;
    float acc[NAL][NB], accw[NAL][NB];
#pragma unroll
    for (int q = 0; q < NAL; ++q)
#pragma unroll
      for (int c = 0; c < NB; ++c) acc[q][c] = accw[q][c] = 0.f;
    // the contributing pairs are recorded for the gradient kernel as
    // j | k << 8 (pcap > 0 only when every slot index fits 8 bits; valid
    // lanes are the low ones of each batch); the count may exceed pcap
    int np = 0;
    unsigned short *prow = pairs + (size_t)i * pcap;
    if (P > 1)
      pair_stream<kPairQFwd>(L.a, P, rc, lane, s_qjk[warp], s_qc2[warp], [&](int j, int k, float c2, bool ok) {
        const unsigned vm = __ballot_sync(0xffffffffu, ok);
        if (ok && np + lane < pcap) prow[np + lane] = (unsigned short)(j | (k << 8));
        np += __popc(vm);
        if (!ok) return;
        const float a = L.a[j].w, b = L.a[k].w;
        const float4 Bj = L.b[j], Bk = L.b[k];
        const float c = c2 > 0.f ? c2 * rsqrtf(c2) : 0.f;
        // costheta = (rij^2 + rik^2 - rjk^2) / (2 rij rik) (wacsf.f90:271-273)
        const float sab = a * a + b * b;
        const float cosv = (sab - c2) * 0.5f * Bj.x * Bk.x;
        const float F = Bj.z * Bk.z * (0.5f * (__cosf(pirc * c) + 1.f));
        const float wjk = Bj.y * Bk.y;
        // exp(-alpha (rij^2 + rik^2 + rjk^2)) as one 2^x (kal = -alpha log2 e)
        const float s3 = sab + c2;
        float EF[NAL];
#pragma unroll
        for (int q = 0; q < NAL; ++q) EF[q] = q < nal ? ex2f(kal[q] * s3) * F : 0.f;
        float basis[NB];
        if constexpr (kB) {
          const float u = fmaf(0.5f, cosv, 0.5f), w = fmaf(-0.5f, cosv, 0.5f);
          const float u2 = u * u, w2 = w * w, uw = u * w;
          basis[0] = w2 * w2;
          basis[1] = uw * w2;
          basis[2] = u2 * w2;
          basis[3] = uw * u2;
          basis[4] = u2 * u2;
        } else {
          ang_powers<NC, STD>(cosv, clam, ciz, basis, nullptr);
        }
#pragma unroll
        for (int q = 0; q < NAL; ++q) {
          const float efw = EF[q] * wjk;
#pragma unroll
          for (int n = 0; n < NB; ++n) {
            acc[q][n] = fmaf(basis[n], EF[q], acc[q][n]);
            accw[q][n] = fmaf(basis[n], efw, accw[q][n]);
          }
        }
      });
    if (lane == 0 && pcap > 0) pcount[i] = np;
#pragma unroll
    for (int q = 0; q < NAL; ++q)
#pragma unroll
      for (int n = 0; n < NB; ++n) {
        const float x = warp_sum(acc[q][n]), y = warp_sum(accw[q][n]);
        if (lane == 0) {
          s_acc[warp][q * NB + n] = x;
          s_acc[warp][NAL * NB + q * NB + n] = y;
        }
      }
    __syncwarp();
    if constexpr (kB) {
      // moments -> the six (1 +- cos)^zeta grids, combination order of ang_powers
      for (int e = lane; e < 2 * NAL * NC; e += 32) {
        const int part = e / (NAL * NC), q = (e / NC) % NAL, cc = e % NC;
        const float *mo = &s_acc[warp][part * NAL * NB + q * NB];
        float v = 0.f;
#pragma unroll
        for (int n = 0; n < 5; ++n) v = fmaf(kBern[cc][n], mo[n], v);
        s_out[warp][part * NAL * NC + q * NC + cc] = v;
      }
      __syncwarp();
    }
    const float *grid = kB ? s_out[warp] : s_acc[warp];
    for (int s = lane; s < nang; s += 32) {
      const int cell = ((sf.ang_code[s] >> 8) & 255) * NC + sf.ang_comb[s];
      const int d = sf.ang_d[s];
      Gi[d] = sf.ang_pref[s] * grid[cell];
      Gi[d + nsf] = sf.ang_pref[s] * grid[NAL * NC + cell];
    }
    __syncwarp();
  }
}

// dE/dG of one atom contracted onto the (alpha, combination) grid,
//   P_q(cos) = sum_c (UA_qc + w_j w_k UB_qc) A_c(cos),
// UA / UB the unweighted and weighted copies (2^(1-zeta) included).  For the
// standard set (A_c = (1 +- cos)^{1,2,4}) P_q is a degree-4 polynomial in
// cos: its coefficients are formed once per atom and a pair evaluates P_q
// and P_q' by one Horner pass; other sets combine the powers A_c directly.
template <int NAL, int NC, bool STD>
struct AngCoef {
  static constexpr bool kPoly = STD && NC == 6;
  float U[2][NAL][kPoly ? 5 : NC];  // [weighting][alpha][coefficient or combination]

  __device__ __forceinline__ void load(const float *su) {
#pragma unroll
    for (int h = 0; h < 2; ++h)
#pragma unroll
      for (int q = 0; q < NAL; ++q) {
        const float *u = su + h * NAL * NC + q * NC;
        if constexpr (kPoly) {
          // (1+x), (1-x), (1+x)^2, (1-x)^2, (1+x)^4, (1-x)^4 expanded in x
          U[h][q][0] = u[0] + u[1] + u[2] + u[3] + u[4] + u[5];
          U[h][q][1] = (u[0] - u[1]) + 2.f * (u[2] - u[3]) + 4.f * (u[4] - u[5]);
          U[h][q][2] = (u[2] + u[3]) + 6.f * (u[4] + u[5]);
          U[h][q][3] = 4.f * (u[4] - u[5]);
          U[h][q][4] = u[4] + u[5];
        } else {
#pragma unroll
          for (int c = 0; c < NC; ++c) U[h][q][c] = u[c];
        }
      }
  }

  // P_q(cos) and dP_q/dcos for every alpha q
  __device__ __forceinline__ void eval(float x, float wjk, const float (&clam)[NC],
                                       const int (&ciz)[NC], float (&Pv)[NAL],
                                       float (&Pd)[NAL]) const {
    if constexpr (kPoly) {
      (void)clam;
      (void)ciz;
#pragma unroll
      for (int q = 0; q < NAL; ++q) {
        float c[5];
#pragma unroll
        for (int m = 0; m < 5; ++m) c[m] = fmaf(wjk, U[1][q][m], U[0][q][m]);
        float p = fmaf(c[4], x, c[3]), d = c[4];
        d = fmaf(d, x, p);
        p = fmaf(p, x, c[2]);
        d = fmaf(d, x, p);
        p = fmaf(p, x, c[1]);
        d = fmaf(d, x, p);
        p = fmaf(p, x, c[0]);
        Pv[q] = p;
        Pd[q] = d;
      }
    } else {
      float A[NC], dAl[NC];
      ang_powers<NC, STD>(x, clam, ciz, A, dAl);
#pragma unroll
      for (int q = 0; q < NAL; ++q) {
        float sp = 0.f, sq = 0.f;
#pragma unroll
        for (int cc = 0; cc < NC; ++cc) {
          const float V = U[0][q][cc] + wjk * U[1][q][cc];
          sp += dAl[cc] * V;
          sq += A[cc] * V;
        }
        Pv[q] = sq;
        Pd[q] = sp;
      }
    }
  }
};

// Gradient of one angular pair's contribution sum_s dE/dG_s G_s(j, k) with
// respect to the positions of slots j and k: vj and vk.  Slot j's records
// (Aj, Bj) come from the caller, which keeps them across a run of pairs that
// share j.  The exponential factor exp(-alpha (rij^2 + rik^2 + rjk^2)) is one
// 2^x with kal = -alpha log2 e.
template <int NAL, int NC, bool STD>
__device__ __forceinline__ void pair_grad(const GLay &L, const float4 &Aj, const float4 &Bj,
                                          int k, float pirc, int nal,
                                          const float (&alv)[NAL], const float (&kal)[NAL],
                                          const float (&clam)[NC],
                                          const int (&ciz)[NC], const AngCoef<NAL, NC, STD> &U,
                                          float3 &vj, float3 &vk) {
  const float4 Ak = L.a[k], Bk = L.b[k];
  const float cx = Aj.x - Ak.x, cy = Aj.y - Ak.y, cz = Aj.z - Ak.z;
  const float c2 = cx * cx + cy * cy + cz * cz;
  const float a = Aj.w, b = Ak.w;
  const float ic = c2 > 0.f ? rsqrtf(c2) : 0.f, c = c2 * ic;
  const float ia = Bj.x, ib = Bk.x;
  const float sab = a * a + b * b, sum2 = sab + c2;
  const float cosv = (sab - c2) * 0.5f * ia * ib;
  const float dcda = ib - cosv * ia, dcdb = ia - cosv * ib, dcdc = -c * ia * ib;
  float sn, cs;
  __sincosf(pirc * c, &sn, &cs);
  const float fcc = 0.5f * (cs + 1.f), dfcc = -0.5f * sn * pirc;
  const float fa = Bj.z, fb = Bk.z, dfa = Bj.w, dfb = Bk.w;
  const float F = fa * fb * fcc;
  float Pv[NAL], Pd[NAL];
  U.eval(cosv, Bj.y * Bk.y, clam, ciz, Pv, Pd);
  float SP = 0.f, SQ = 0.f, SU = 0.f;
#pragma unroll
  for (int q = 0; q < NAL; ++q) {
    const float E = q < nal ? ex2f(kal[q] * sum2) : 0.f;
    SP += E * Pd[q];
    SQ += E * Pv[q];
    SU += alv[q] * E * Pv[q];
  }
  // dG/da = E [A' dcos/da F + A (-2 alpha a F + fc'(a) fc(b) fc(c))], etc.
  const float S1 = F * (SP * dcda - 2.f * SU * a) + SQ * (dfa * fb * fcc);
  const float S2 = F * (SP * dcdb - 2.f * SU * b) + SQ * (fa * dfb * fcc);
  const float S3 = F * (SP * dcdc - 2.f * SU * c) + SQ * (fa * fb * dfcc);
  const float s1 = S1 * ia, s2 = S2 * ib, s3 = S3 * ic;
  vj = make_float3(s1 * Aj.x + s3 * cx, s1 * Aj.y + s3 * cy, s1 * Aj.z + s3 * cz);
  vk = make_float3(s2 * Ak.x - s3 * cx, s2 * Ak.y - s3 * cy, s2 * Ak.z - s3 * cz);
}

// Slot gradients g_q = sum_d dE/dG_id dG_id/dp_q of each atom, the force
// scatter and the per-atom virial.
//  - radial terms: lanes own slots; per SF one broadcast record
//    (kx, rs, dE/dG_d, dE/dG_{d+nsf}) staged per atom;
//  - angular pairs: the pair list the forward kernel recorded is split into
//    32 contiguous chunks, one per lane.  The list is j-major, so a lane's
//    consecutive pairs share slot j: its j-side gradient stays in registers
//    and is added to shared memory only when j changes (a few times per
//    atom); the k side is added per pair by shared-memory atomics.  Atoms
//    whose list overflowed re-enumerate their pairs (pair_stream) and sum
//    the j side by a segmented warp scan.
template <int NAL, int NC, bool STD>
__global__ void __launch_bounds__(32 * kWarpsPerBlock, (grp_bwd_blocks<NAL, NC, STD>()))
    k_wacsf_bwd_grp(int N, int i0, int cap, int capS, const int *__restrict__ cnt,
                    const double4 *__restrict__ xyzr, const int *__restrict__ nj,
                    const double4 *__restrict__ apos, const float4 *__restrict__ d32,
                    const float *__restrict__ w32, const SFT<float> *__restrict__ sfg,
                    const float *__restrict__ dedg, double *__restrict__ force,
                    double *__restrict__ wvir, const unsigned short *__restrict__ pairs,
                    const int *__restrict__ pcount, int pcap, int *__restrict__ flags) {
  (void)xyzr;
  (void)apos;
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ int s_qjk[kWarpsPerBlock][kPairQBwd + 32];  // ring + the lanes' spare entries
  __shared__ float s_qc2[kWarpsPerBlock][kPairQBwd + 32];
  __shared__ float s_u[kWarpsPerBlock][2 * NAL * NC];
  load_table<float>(smraw, sfg);
  const SFT<float> &sf = *reinterpret_cast<const SFT<float> *>(smraw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nal = sf.nalpha, D = sf.D, nsf = sf.nsf, nrad = sf.nrad, nang = sf.nang;
  const GLay L = grp_carve(smraw, warp, capS, sf.nrc, D, nrad, false);
  const int rci = nang > 0 ? sf.ang_grp_rc[0] : 0;
  const float rc = sf.rc_val[rci], pirc = sf.pi_over_rc[rci];
  float alv[NAL], kal[NAL], clam[NC];
  int ciz[NC];
#pragma unroll
  for (int q = 0; q < NAL; ++q) {
    alv[q] = q < nal ? sf.alpha_val[q] : 0.f;
    kal[q] = -alv[q] * kLog2e;
  }
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    clam[c] = sf.comb_lam[c];
    ciz[c] = sf.comb_iz[c];
  }
  bool bad = false;  // a slot-gradient term outside the fixed-point range
  for (int i = blockIdx.x * kWarpsPerBlock + warp; i < N; i += gridDim.x * kWarpsPerBlock) {
    const int P = grp_stage(L, sf, i, cap, capS, lane, rci, cnt, d32, w32, true);
    for (int d = lane; d < D; d += 32) L.dg[d] = dedg[(size_t)i * D + d];
    for (int e = lane; e < 2 * NAL * NC; e += 32) s_u[warp][e] = 0.f;
    __syncwarp();
    // per-atom radial records: (kx, rs, dE/dG_d, dE/dG_{d+nsf})
    for (int s = lane; s < nrad; s += 32) {
      const int d = sf.rad_d[s];
      L.rco[s] = make_float4(-sf.rad_alpha[s] * kLog2e, sf.rad_rs[s], L.dg[d], L.dg[d + nsf]);
    }
    // dE/dG contracted onto the (alpha, combination) grid: one SF per lane
    for (int s = lane; s < nang; s += 32) {
      const int cell = ((sf.ang_code[s] >> 8) & 255) * NC + sf.ang_comb[s];
      const int d = sf.ang_d[s];
      atomicAdd(&s_u[warp][cell], sf.ang_pref[s] * L.dg[d]);
      atomicAdd(&s_u[warp][NAL * NC + cell], sf.ang_pref[s] * L.dg[d + nsf]);
    }
    __syncwarp();
    // radial terms: lanes own slots.  d/dr [ex fc] = ex (fc' - 2 alpha u fc),
    // -2 alpha = 2 ln2 kx
    for (int q = lane; q < P; q += 32) {
      const float4 aq = L.a[q], bq = L.b[q];
      const float r = aq.w, w = bq.y;
      float S = 0.f;
      if (sf.nrc == 1) {
        const float f = bq.z, df = bq.w;
#pragma unroll 4
        for (int s = 0; s < nrad; ++s) {
          const float4 c = L.rco[s];
          const float u = r - c.y;
          const float ex = ex2f(c.x * (u * u));
          const float t = fmaf(c.x * kTwoLn2 * u, f, df);
          S = fmaf(fmaf(c.w, w, c.z) * ex, t, S);
        }
      } else {
        for (int s = 0; s < nrad; ++s) {
          const float4 c = L.rco[s];
          const int rr = sf.rad_rc[s];
          const float f = L.fc[rr * capS + q], df = L.dfc[rr * capS + q];
          const float u = r - c.y;
          const float ex = ex2f(c.x * (u * u));
          const float t = fmaf(c.x * kTwoLn2 * u, f, df);
          S = fmaf(fmaf(c.w, w, c.z) * ex, t, S);
        }
      }
      const float ir = S / r;
      slot_set(L, q, ir * aq.x, ir * aq.y, ir * aq.z, bad);  // every slot's first write
    }
    __syncwarp();
    if (nang > 0) {
      AngCoef<NAL, NC, STD> U;
      U.load(s_u[warp]);
      const int np = pcap > 0 ? pcount[i] : -1;
      if (np >= 0 && np <= pcap) {
        // the pairs the descriptor kernel found: lane-contiguous chunks
        const unsigned short *prow = pairs + (size_t)i * pcap;
        const int C = (np + 31) >> 5;
        const int p0 = lane * C, pe = min(np, p0 + C);
        int nxt = p0 < pe ? (int)prow[p0] : 0;
        int cur = -1;
        float gjx = 0.f, gjy = 0.f, gjz = 0.f;
        float4 Aj = make_float4(0.f, 0.f, 0.f, 0.f), Bj = Aj;  // slot cur's records
        for (int t = 0; t < C; ++t) {
          const int p = p0 + t;
          const int jk = nxt;
          if (p + 1 < pe) nxt = (int)prow[p + 1];  // next pair's entry, loaded ahead
          if (p < pe) {
            const int j = jk & 0xff, k = jk >> 8;
            if (j != cur) {
              if (cur >= 0) slot_add(L, cur, gjx, gjy, gjz, bad);
              cur = j;
              gjx = gjy = gjz = 0.f;
              Aj = L.a[j];
              Bj = L.b[j];
            }
            float3 vj, vk;
            pair_grad<NAL, NC, STD>(L, Aj, Bj, k, pirc, nal, alv, kal, clam, ciz, U, vj, vk);
            gjx += vj.x;
            gjy += vj.y;
            gjz += vj.z;
            slot_add(L, k, vk.x, vk.y, vk.z, bad);
          }
        }
        if (cur >= 0) slot_add(L, cur, gjx, gjy, gjz, bad);
      } else if (P > 1) {
        pair_stream<kPairQBwd>(L.a, P, rc, lane, s_qjk[warp], s_qc2[warp], [&](int j, int k, float c2, bool ok) {
          (void)c2;
          float3 vj, vk;
          pair_grad<NAL, NC, STD>(L, L.a[j], L.b[j], k, pirc, nal, alv, kal, clam, ciz, U, vj, vk);
          float vx = ok ? vj.x : 0.f, vy = ok ? vj.y : 0.f, vz = ok ? vj.z : 0.f;
          // slot j: equal j values are contiguous lanes of the batch, summed
          // by a segmented scan whose last lane adds the run
          const unsigned run = __match_any_sync(0xffffffffu, ok ? j : 0x10000 + lane);
          const int first = __ffs(run) - 1, last = 31 - __clz(run);
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const float tx = __shfl_up_sync(0xffffffffu, vx, o);
            const float ty = __shfl_up_sync(0xffffffffu, vy, o);
            const float tz = __shfl_up_sync(0xffffffffu, vz, o);
            if (lane - o >= first) {
              vx += tx;
              vy += ty;
              vz += tz;
            }
          }
          if (ok && lane == last) slot_add(L, j, vx, vy, vz, bad);
          if (ok) slot_add(L, k, vk.x, vk.y, vk.z, bad);
        });
      }
    }
    __syncwarp();
    // forces by scatter: with g_q = sum_d dE/dG_id dG_id/dp_q and the
    // translation invariance of G_i, atom i receives +sum_q g_q and slot q's
    // atom -g_q (FP64 atomics; F is zeroed before the launch)
    float W[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    float fx = 0.f, fy = 0.f, fz = 0.f;
    for (int q = lane; q < P; q += 32) {
      const int2 *w = reinterpret_cast<const int2 *>(L.g6 + 6 * q);
      const float gx = fx_value(w[0]), gy = fx_value(w[1]), gz = fx_value(w[2]);
      const int j = nj[(size_t)i * cap + q];
      atomicAdd(force + (size_t)j * 3 + 0, -(double)gx);
      atomicAdd(force + (size_t)j * 3 + 1, -(double)gy);
      atomicAdd(force + (size_t)j * 3 + 2, -(double)gz);
      fx += gx;
      fy += gy;
      fz += gz;
      const float4 aq = L.a[q];
      const float d3[3] = {aq.x, aq.y, aq.z};
      const float g3[3] = {gx, gy, gz};
#pragma unroll
      for (int aa = 0; aa < 3; ++aa)
#pragma unroll
        for (int bb = 0; bb < 3; ++bb) W[aa * 3 + bb] += d3[aa] * g3[bb];
    }
    fx = warp_sum<float>(fx);
    fy = warp_sum<float>(fy);
    fz = warp_sum<float>(fz);
    if (lane == 0) {  // atom i's own force: index i0 + i of the whole batch
      atomicAdd(force + (size_t)(i0 + i) * 3 + 0, (double)fx);
      atomicAdd(force + (size_t)(i0 + i) * 3 + 1, (double)fy);
      atomicAdd(force + (size_t)(i0 + i) * 3 + 2, (double)fz);
    }
    // per-atom virial in FP32 (a sum over its own slots); the sums over
    // atoms are FP64 (k_struct_reduce)
#pragma unroll
    for (int t = 0; t < 9; ++t) W[t] = warp_sum<float>(W[t]);
    if (lane < 9) {
      float v = 0.f;
#pragma unroll
      for (int t = 0; t < 9; ++t)
        if (lane == t) v = W[t];
      wvir[(size_t)i * 9 + lane] = (double)v;
    }
    __syncwarp();
  }
  if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(flags, kFlagForceRange);
}

// Kernel pointers of every (NAL, NC) instantiation.
template <int NAL, int NC, bool STD = false>
struct GrpPair {
  static constexpr auto fwd = k_wacsf_fwd_grp<NAL, NC, STD>;
  static constexpr auto bwd = k_wacsf_bwd_grp<NAL, NC, STD>;
};

using GrpFwd = decltype(&k_wacsf_fwd_grp<1, 2, false>);
using GrpBwd = decltype(&k_wacsf_bwd_grp<1, 2, false>);

template <int NAL>
__host__ inline void pick_nc(int nc, bool std6, GrpFwd *f, GrpBwd *b) {
  switch (nc) {
    case 2: *f = GrpPair<NAL, 2>::fwd; *b = GrpPair<NAL, 2>::bwd; break;
    case 4: *f = GrpPair<NAL, 4>::fwd; *b = GrpPair<NAL, 4>::bwd; break;
    case 6:
      if (std6) { *f = GrpPair<NAL, 6, true>::fwd; *b = GrpPair<NAL, 6, true>::bwd; }
      else { *f = GrpPair<NAL, 6>::fwd; *b = GrpPair<NAL, 6>::bwd; }
      break;
    default: *f = GrpPair<NAL, 8>::fwd; *b = GrpPair<NAL, 8>::bwd; break;
  }
}

// The grouped kernels for a model, or false when it does not qualify.
__host__ inline bool grouped_kernels(const SFT<float> &t, GrpFwd *f, GrpBwd *b) {
  if (t.fast_nal == 0 || t.fast_nc == 0) return false;
  const bool std6 = t.std6 && t.fast_nc == 6;
  switch (t.fast_nal) {
    case 1: pick_nc<1>(t.fast_nc, std6, f, b); break;
    case 2: pick_nc<2>(t.fast_nc, std6, f, b); break;
    default: pick_nc<4>(t.fast_nc, std6, f, b); break;
  }
  return true;
}
