// Phase 2 in packed 16-bit lanes with the DPX add-max instructions.
//
// Same recurrence and tie rules as sw.cu (the reference kernel's,
// src/smithWaterman.cu:510-645 and 911-1026).  Two passes share the
// layout:
//   score pass   (TRACE = false): the exact maximum score of a pair, for
//                best-per-read selection (with the LCS pass's suffix values,
//                stopped once the score is settled or provably too low to
//                be picked);
//   trace pass   (TRACE = true):  for the printed pairs, the first
//                row-major maximum and 4-bit directions streamed to global
//                scratch; sw_walk_kernel then walks the reference's
//                traceback, one thread per pair.
//
// Encoding.  Each cell is kept as Hx = 16*H + code + B, where code is the
// one-hot direction the reference would store (NONE 8, DIAG 4, UP 2,
// LEFT 1) and B a bias that keeps every candidate non-negative.  The
// candidates enter one max as
//     DIAG: 16*(H[i-1][j-1] + s) + 4 + B
//     UP:   16*(H[i-1][j] + pen) + 2 + B
//     LEFT: 16*(H[i][j-1] + pen) + 1 + B
//     NONE: 8 + B   (H = 0)
// so the max yields H and, on equal H, the reference's precedence
// NONE > DIAG > UP > LEFT of its strict '>' updates.  A neighbour's gap
// penalty is gap_ext when its own code is UP (for the cell below) or LEFT
// (for the cell to the right), else gap_open; bits 1 and 0 of Hx give that:
//     xU = (Hx & ~15) + (Hx & 2) * 8 (e - o)     UP candidate  = xU + 16 o + 2
//     xL = (Hx & ~15) + (Hx & 1) * 16 (e - o)    LEFT candidate = xL + 16 o + 1
// Two pairs share one 32-bit register (low / high 16 bits).
//
// Layout.  A warp holds 32/G groups of G lanes; each group runs two pairs
// packed in the 16-bit halves.  Lane t of a group owns query rows
// t*RPL+1 .. t*RPL+RPL and sweeps the window one column behind lane t-1 (an
// anti-diagonal wavefront of row strips); the bottom row's UP candidate and
// H pass down with two shuffles per column.  The substitution score comes
// from a per-row profile register pair selected by one byte permute per
// cell.  Rows past the query get an all-mismatch profile: with negative
// mismatch and gap penalties their cells stay strictly below the maximum of
// the rows above, so the score pass can keep a single running maximum per
// lane.  The trace pass keeps the first maximum of every row (packed compare:
// 16-bit integer patterns compared as non-negative half floats, whose order
// they share, then two selects).
//
// Preconditions (checked by fast_params_ok and per pair by the pair kernel;
// other pairs take sw.cu): query and window bytes in {A,C,G,T,a,c,g,t},
// window length = R, mismatch, gap_open, gap_ext < 0, gap_ext >= gap_open,
// |16*score+4| < 128, 16 * match * Q + B stays below 0x7C00.
#pragma once

#include <string.h>

#include <type_traits>
#include "internal.h"

namespace swift {
namespace {

// warps per block: small blocks, because a block holds its SM slot until
// its last warp ends and warps that stop early end at different steps
constexpr int kPkWarps = 2;

__device__ __forceinline__ uint32_t base_class(uint32_t c) {
  uint32_t u = c & 0xDFu;
  return u == 'C' ? 1u : u == 'G' ? 2u : u == 'T' ? 3u : 0u;
}

// per-half 0xFFFF where a > b, for non-negative 16-bit integers below 0x7C00
__device__ __forceinline__ uint32_t gt_mask(uint32_t a, uint32_t b) {
  uint32_t d;
  asm("set.gt.u32.f16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
  return d;
}

// byte permute with sign replication (PTX prmt, default mode)
__device__ __forceinline__ uint32_t prmt(uint32_t a, uint32_t b, uint32_t s) {
  uint32_t d;
  asm("prmt.b32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(s));
  return d;
}

// a * b + c as an integer multiply-add: with b a runtime value the compiler
// cannot fold, it stays one (FMA-pipe) instruction instead of becoming a
// shift-add or an add on the ALU pipe
__device__ __forceinline__ uint32_t mad_u32(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t d;
  asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
  return d;
}

__device__ __forceinline__ uint32_t sel(uint32_t m, uint32_t a, uint32_t b) {
  return (a & m) | (b & ~m);
}

// Direction scratch of the trace pass, per group (two pairs): per lane ln
// the words of consecutive wavefront steps, the kDirWords words of a step
// side by side,
//     region[(ln * steps8 + step) * kDirWords + w],  steps8 = steps rounded up to 8,
// so a block of 4 steps is one 16 * kDirWords-byte store and a traceback,
// which moves one step back on most cells, reads neighbouring words of one
// stream per lane.  A word holds up to 8 rows x 2 pairs x 2 bits, its last
// row lowest: with n rows in the word (8, or what is left of the lane's
// rows), bits 2 * (n - 1 - (k & 7)) (first pair) and 16 + the same (second
// pair) of row k are 2 for UP, 1 for LEFT and 0 for DIAG or NONE (NONE is
// the cell with H = 0, which the traceback knows from the scores).
// first-maximum tags of the trace pass (see packed_item)
constexpr uint32_t kTagOld = 0x000F000Fu;
constexpr int kTagWindow = 12;

template <int RPL>
struct DirLayout {
  static constexpr int kWords = (RPL + 7) / 8;  // words per lane and step
};
__host__ __device__ constexpr int steps8(int R, int G) { return (R + G - 1 + 7) & ~7; }

// VAR: pairs of one launch may differ in length (a.q_len / a.r_len per pair):
// rows past a pair's query are all-mismatch rows as usual, the warp sweeps
// the longest window of its pairs, and columns past a pair's own window are
// kept out of its first-maximum bookkeeping (their cells are computed but
// never reach the maximum, the traceback or the result).
template <int G, int RPL, bool TRACE, bool VAR>
__device__ __forceinline__ void packed_item(const FastArgs& a, const int64_t warp, const int64_t nlist,
                                            uint32_t* wsel_all, const int wib, const int lane) {
  constexpr int kGroups = 32 / G;      // groups per warp
  constexpr int kPairs = 2 * kGroups;  // pairs per warp
  constexpr int kNW = DirLayout<RPL>::kWords;
  const int g = lane / G, sl = lane % G;
  const int64_t base = warp * kPairs + 2 * g;
  const int32_t* list = a.list + a.list_offset;
  const bool has0 = base < nlist, has1 = base + 1 < nlist;
  const int32_t p0 = has0 ? list[base] : list[nlist - 1];
  const int32_t p1 = has1 ? list[base + 1] : p0;
  const int Q0 = VAR ? a.q_len[p0] : a.Q, Q1 = VAR ? a.q_len[p1] : a.Q;
  // per-pair windows when r_len is given, else every window is a.R long
  const bool var_r = VAR && a.r_len != nullptr;
  const int R0 = var_r ? a.r_len[p0] : a.R, R1 = var_r ? a.r_len[p1] : a.R;
  // columns the warp sweeps
  const int R = var_r ? (int)__reduce_max_sync(0xffffffffu, (unsigned)max(R0, R1)) : a.R;
  const char* q0 = a.q + (int64_t)p0 * a.q_stride;
  const char* q1 = a.q + (int64_t)p1 * a.q_stride;
  const char* w0 = a.w + (int64_t)p0 * a.w_stride;
  const char* w1 = a.w + (int64_t)p1 * a.w_stride;
  uint32_t* wsel = wsel_all + (wib * kGroups + g) * (a.R + 1);
  for (int c = sl; c < R; c += G) {
    uint32_t s0 = (!VAR || c < R0) ? base_class((uint8_t)w0[c]) : 0u;
    uint32_t s1 = (!VAR || c < R1) ? base_class((uint8_t)w1[c]) : 0u;
    wsel[c + 1] = s0 | ((s0 | 8u) << 4) | ((4u + s1) << 8) | (((4u + s1) | 8u) << 12);
  }
  __syncwarp();
  const uint32_t B = (uint32_t)a.bias;
  const uint32_t BB = B | (B << 16);
  const uint32_t B8 = BB + 0x00080008u;
  // per-half subtraction as one 32-bit add: every half it meets is at least
  // B > |constant|, so no borrow crosses between the halves
  const uint32_t CU = (uint32_t)((int32_t)(16 * a.gap_open + 2) * 65537);
  const uint32_t CL = (uint32_t)((int32_t)(16 * a.gap_open + 1) * 65537);
  const uint32_t KU = (uint32_t)(8 * (a.gap_ext - a.gap_open));
  const uint32_t KL = (uint32_t)(16 * (a.gap_ext - a.gap_open));
  const uint32_t sm = (uint32_t)(uint8_t)(int8_t)(16 * a.match + 4);
  const uint32_t sx = (uint32_t)(uint8_t)(int8_t)(16 * a.mismatch + 4);
  const uint32_t all_x = sx * 0x01010101u;
  uint32_t prof0[RPL], prof1[RPL], h16p[RPL], xl[RPL];
  uint32_t bestv[TRACE ? RPL : 1], bestc[TRACE ? RPL : 1];
#pragma unroll
  for (int k = 0; k < RPL; ++k) {
    const int i = sl * RPL + k;
    // past the query: mismatch everywhere
    prof0[k] = i < Q0 ? all_x ^ ((sm ^ sx) << (8 * base_class((uint8_t)q0[i]))) : all_x;
    prof1[k] = i < Q1 ? all_x ^ ((sm ^ sx) << (8 * base_class((uint8_t)q1[i]))) : all_x;
    h16p[k] = BB;  // H[i][0] = 0
    xl[k] = BB;    // column 0 is NONE
    if (TRACE) {
      bestv[k] = BB | kTagOld;  // H = 0 cells (key B + tag < B + 15) never replace it
      bestc[k] = 0;
    }
  }
  if (!TRACE) bestv[0] = BB;
  const int S8 = steps8(a.R, G);  // the launch's layout (the walk's too)
  uint32_t* dirs = nullptr;
  if (TRACE) dirs = a.dirs + ((warp * kGroups + g) * G + sl) * (int64_t)kNW * S8;
  uint32_t send_u = BB, send_h = BB, diag = BB;
  // one wavefront step; acc receives the step's direction words.  `full`
  // (std::true_type) marks a step whose columns lie inside the window on
  // every lane of the group: the range check and its merges drop out.
  // tag: the step's first-maximum tag (trace pass), both halves.  `masked`
  // (VAR with per-pair windows): some pair of the warp may have its window
  // end before the step's columns, so the first-maximum keys are masked.
  auto step = [&](const int s, uint32_t* acc, auto full, auto masked, const uint32_t tag) {
    constexpr bool kFull = decltype(full)::value;
    constexpr bool kMasked = decltype(masked)::value;
    uint32_t up = __shfl_up_sync(0xffffffffu, send_u, 1, G);
    const uint32_t rh = __shfl_up_sync(0xffffffffu, send_h, 1, G);
    if (sl == 0) up = BB;  // row 0: H = 0, NONE
    const int j = s - sl + 1;
#pragma unroll
    for (int w = 0; w < kNW; ++w) acc[w] = 0;
    if (kFull || (j >= 1 && j <= R)) {
      const uint32_t ws = wsel[j];
      // VAR: halves whose window ends before column j
      const uint32_t cm = kMasked && var_r ? ((j <= R0 ? 0x0000FFFFu : 0u) | (j <= R1 ? 0xFFFF0000u : 0u)) : ~0u;
      uint32_t dg = diag;
      uint32_t hpair = 0;  // score pass: even row waiting for its odd partner
#pragma unroll
      for (int k = 0; k < RPL; ++k) {
        const uint32_t sc = prmt(prof0[k], prof1[k], ws);
        // DIAG (signed substitution score) against LEFT first: neither waits
        // for the row above, which then enters one three-way max with the
        // NONE floor (the candidates' plain adds issue on the FMA pipe)
        const uint32_t dl = __viaddmax_s16x2(dg, sc, xl[k] + CL);
        const uint32_t hx = __vimax3_s16x2(dl, up + CU, B8);
        dg = h16p[k];
        const uint32_t h16 = hx & 0xFFF0FFF0u;
        h16p[k] = h16;
        const uint32_t bu = hx & 0x00020002u, bl = hx & 0x00010001u;  // UP, LEFT
        up = bu * KU + h16;
        xl[k] = bl * KL + h16;
        if (TRACE) {
          // first maximum of the row: the key's tag makes an earlier step of
          // the window win a tie, and the window's last best keeps tag 15
          // (one add-max; both operands non-negative)
          if (VAR && kMasked && var_r)
            bestv[k] = __vimax_s16x2_relu(bestv[k], (h16 + tag) & cm);
          else
            bestv[k] = __viaddmax_s16x2(h16, tag, bestv[k]);
          // the UP and LEFT bits of each half's code enter the word by
          // Horner's rule (word * 4 + bits; 8 rows of 2 bits fill a half
          // without crossing into the other), with the masks above, as two
          // FMA-pipe multiply-adds
          if ((k & 7) == 0) {
            acc[k >> 3] = mad_u32(bl, a.one, bu);
          } else {
            acc[k >> 3] = mad_u32(acc[k >> 3], a.four, bu);
            acc[k >> 3] = mad_u32(bl, a.one, acc[k >> 3]);
          }
        } else if (k & 1) {
          bestv[0] = __vimax3_s16x2_relu(bestv[0], hpair, h16);
        } else if (k == RPL - 1) {
          bestv[0] = __vimax_s16x2_relu(bestv[0], h16);
        } else {
          hpair = h16;
        }
      }
      send_u = up;
      send_h = h16p[RPL - 1];
    }
    diag = sl == 0 ? BB : rh;
  };
  const int steps = R + G - 1;
  // VAR: columns up to r_min lie inside every pair's window (steps s with
  // s + 1 <= r_min need no masks)
  const int r_min = var_r ? (int)__reduce_min_sync(0xffffffffu, (unsigned)min(R0, R1)) : R;
  // Trace pass, first maximum of each row: the key of a cell is h16 + tag,
  // tag = 14 - (its step's offset in a window of kTagWindow steps), so one
  // max keeps the largest H and, among equal H, the earliest step of the
  // window.  At the window's end the halves whose tag is not 15 took a new
  // maximum there: their column (stored + 32, so no half borrows) is
  // recovered from the tag and the tag is set to 15, above every tag a
  // later window can give an equal H.
  int sw = 0;  // first step of the current window
  auto flush_window = [&]() {
    if (!TRACE) return;
    const uint32_t base = (uint32_t)(sw - sl + 1 + 14 + 32) * 0x00010001u;
#pragma unroll
    for (int k = 0; k < (TRACE ? RPL : 0); ++k) {
      const uint32_t tg = bestv[k] & kTagOld;
      // tags 3..15 shifted to the half exponent: normal numbers, same order
      const uint32_t m = gt_mask(kTagOld << 10, tg << 10);
      bestc[k] = sel(m, base - tg, bestc[k]);
      bestv[k] |= kTagOld;
    }
  };
  // Early stop (the trace of each read's candidate, the exact score pass),
  // from the suffix LCS values of the LCS bound pass.  After step
  // s = kSufSteps * m + G - 1 every cell not computed yet lies right of
  // column kSufSteps * m.  Unrolling the recurrence from such a cell back
  // to its origin gives a chain of cells that starts either with H = 0
  // among the cells not computed (its matches then lie in columns
  // > kSufSteps * m) or at a computed cell f = (i, j) one of whose
  // successors is not computed (its matches then lie in rows > i and
  // columns > j).  Mismatches and gaps only lower a chain, so the cell's H
  // is at most
  //     max(match * L_m, H(f) + match * min(Q - i, L_m)),
  // L_m = LCS(query, window columns kSufSteps * m + 1 .. R).  Those f are
  // each row's current cell and, for the last row of a lane, the cell one
  // column back, which the lane below holds as its diagonal input.  Once
  // the bound is below the pair's maximum so far, no cell left can be (or
  // tie) its first maximum and the traceback never reaches one.  The score
  // pass needs only the maximum, so a bound equal to it is enough, and with
  // a.cand a pair also stops once the bound and its maximum so far are both
  // below T, the least score that could still make it its group's pick
  // (its candidate's score, + 1 after the candidate in group order): its
  // maximum so far, reported, stays below T as its true score does.  Every
  // value stays at most 16 * match * Q + B (H(f) <= match * i).
  const bool lcs_on = a.lsuf != nullptr && !var_r;
  uint32_t lnext0 = 0, lnext1 = 0;  // L_m of the next check, loaded ahead
  uint32_t thr = 0;                 // score pass: 16 * T + B per half, 0: none
  if (lcs_on) {
    lnext0 = a.lsuf[(int64_t)p0 * kSufBlocks + 1];
    lnext1 = a.lsuf[(int64_t)p1 * kSufBlocks + 1];
    if (!TRACE && a.cand) {
      const int32_t c0 = a.cand[p0], c1 = a.cand[p1];
      const uint32_t t0 = (uint32_t)(a.aln[c0].score + (p0 > c0 ? 1 : 0));
      const uint32_t t1 = (uint32_t)(a.aln[c1].score + (p1 > c1 ? 1 : 0));
      thr = (B + 16u * t0) | ((B + 16u * t1) << 16);
    }
  }
  auto lcs_stop = [&](const int m) -> bool {
    const uint32_t L0 = lnext0, L1 = lnext1;
    if (m + 1 < kSufBlocks) {
      lnext0 = a.lsuf[(int64_t)p0 * kSufBlocks + m + 1];
      lnext1 = a.lsuf[(int64_t)p1 * kSufBlocks + m + 1];
    }
    // the pair's maximum so far, 16 * score + B per half
    uint32_t v = bestv[0];
#pragma unroll
    for (int k = 1; k < (TRACE ? RPL : 1); ++k) v = __vimax_s16x2_relu(v, bestv[k]);
#pragma unroll
    for (int d = G / 2; d > 0; d >>= 1) v = __vimax_s16x2_relu(v, __shfl_xor_sync(0xffffffffu, v, d, G));
    v &= 0xFFF0FFF0u;
    const uint32_t M16 = 16u * (uint32_t)a.match;
    // per half: nothing left can raise the maximum (trace pass: or tie it),
    // or nothing, computed or left, reaches the threshold
    auto settled = [&](uint32_t f, uint32_t b, uint32_t t) {
      return TRACE ? f < b : (f <= b || (f < t && b < t));
    };
    auto below = [&](uint32_t f) {
      return (!has0 || settled(f & 0xFFFFu, v & 0xFFFFu, thr & 0xFFFFu)) &&
             (!has1 || settled(f >> 16, v >> 16, thr >> 16));
    };
    uint32_t F = (B + M16 * L0) | ((B + M16 * L1) << 16);
    // chains that start among the cells not computed first (cheap, and
    // false until the window's rest holds too few matches)
    if (!__all_sync(0xffffffffu, below(F))) return false;
    // 16 * match * (rows below row k of the lane) per half, signed: row k
    // has a - k below it (a lane wholly past the query starts at -1), so
    // min(that, 16 * match * L) clamped at 0 is the chain's largest gain
    const int a0 = max(Q0 - sl * RPL - 1, -1), a1 = max(Q1 - sl * RPL - 1, -1);
    const uint32_t L16 = (M16 * L0) | ((M16 * L1) << 16);
    const uint32_t step_dn = (0x10000u - M16) * 0x00010001u;  // -16 * match, both halves
    constexpr uint32_t kNoFloor = 0x80008000u;                 // max(x, this) = x
    uint32_t A = ((M16 * (uint32_t)a0) & 0xFFFFu) | ((M16 * (uint32_t)a1) << 16);
    // the lane above's last row (row 0 for lane 0, H = 0) has a + 1 below it
    F = __viaddmax_s16x2(diag, __vimin_s16x2_relu(__viaddmax_s16x2(A, M16 * 0x00010001u, kNoFloor), L16), F);
#pragma unroll
    for (int k = 0; k < RPL; ++k) {
      F = __viaddmax_s16x2(h16p[k], __vimin_s16x2_relu(A, L16), F);
      A = __viaddmax_s16x2(A, step_dn, kNoFloor);
    }
#pragma unroll
    for (int d = G / 2; d > 0; d >>= 1) F = __vimax_s16x2_relu(F, __shfl_xor_sync(0xffffffffu, F, d, G));
    return __all_sync(0xffffffffu, below(F));
  };
  // steps in blocks of 4: the trace pass keeps a block's direction words in
  // registers and writes each word index as one 16-byte store
  uint32_t hist[TRACE ? 4 : 1][kNW];
  int s_end = steps;  // wavefront steps the warp ran
  for (int s0 = 0; s0 < steps; s0 += 4) {
    // steps s0..s0+3 have 1 <= j <= R on every lane when s0 >= G - 1 and
    // s0 + 3 <= R - 1 (then also s0 + 3 < steps)
    // tag of step s0 + u: 14 - (its offset in the window)
    const uint32_t tag0 = (uint32_t)(14 - (s0 - sw)) * 0x00010001u;
    if (s0 >= G - 1 && s0 + 3 <= R - 1 && (!VAR || s0 + 4 <= r_min)) {
#pragma unroll
      for (int u = 0; u < 4; ++u)
        step(s0 + u, hist[TRACE ? u : 0], std::true_type(), std::false_type(),
             tag0 - (uint32_t)u * 0x00010001u);
    } else if (VAR && s0 >= G - 1 && s0 + 3 <= R - 1) {
#pragma unroll
      for (int u = 0; u < 4; ++u)
        step(s0 + u, hist[TRACE ? u : 0], std::true_type(), std::true_type(),
             tag0 - (uint32_t)u * 0x00010001u);
    } else {
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (s0 + u < steps)
          step(s0 + u, hist[TRACE ? u : 0], std::false_type(), std::true_type(),
               tag0 - (uint32_t)u * 0x00010001u);
    }
    if (TRACE) {
      // words s0 * kNW .. (s0 + 4) * kNW - 1 of the lane, step-major (words
      // past the last step are never read)
#pragma unroll
      for (int q = 0; q < kNW; ++q) {
        const int f = 4 * q;
        const uint4 v = make_uint4(hist[f / kNW][f % kNW], hist[(f + 1) / kNW][(f + 1) % kNW],
                                   hist[(f + 2) / kNW][(f + 2) % kNW], hist[(f + 3) / kNW][(f + 3) % kNW]);
        __stcg(reinterpret_cast<uint4*>(dirs + (int64_t)s0 * kNW) + q, v);
      }
      if (s0 + 4 - sw == kTagWindow) {
        flush_window();
        sw = s0 + 4;
      }
    }
    // early-stop test after steps s = kSufSteps * m + G - 1 ((G - 1) % 4 ==
    // 3, so such an s ends a block)
    const int s = s0 + 3;
    if (lcs_on && s >= kSufSteps + G - 1 && ((s - (G - 1)) & (kSufSteps - 1)) == 0 &&
        lcs_stop((s - (G - 1)) / kSufSteps)) {
      s_end = s + 1;
      break;
    }
  }
  if (a.cells_done) {
    // cells of the warp's pairs inside the columns every lane finished
    const int cols = min(s_end - (G - 1), R);
    const uint32_t c = sl != 0 ? 0u
                               : (has0 ? (uint32_t)(min(cols, R0) * Q0) : 0u) +
                                     (has1 ? (uint32_t)(min(cols, R1) * Q1) : 0u);
    const uint32_t warp_cells = __reduce_add_sync(0xffffffffu, c);
    if (lane == 0 && warp_cells) atomicAdd(a.cells_done, (unsigned long long)warp_cells);
  }
  flush_window();
  if (!TRACE) {
    // maximum of the group, per packed pair
    uint32_t v = bestv[0];
#pragma unroll
    for (int d = G / 2; d > 0; d >>= 1) v = __vimax_s16x2_relu(v, __shfl_xor_sync(0xffffffffu, v, d, G));
    if (sl == 0) {
      const uint32_t v0 = v & 0xFFFFu, v1 = v >> 16;
      if (has0) a.aln[p0].score = v0 > B ? (int)((v0 - B) >> 4) : 0;
      if (has1) a.aln[p1].score = v1 > B ? (int)((v1 - B) >> 4) : 0;
    }
    return;
  }
  // first maximum in row-major order, per packed pair
  int32_t cellm[2] = {0, 0}, scorem[2] = {0, 0};
#pragma unroll
  for (int hp = 0; hp < 2; ++hp) {
    const int sh = 16 * hp;
    uint32_t bv = 0, bc = 0, br = 0x7fffffffu;
    const int nrows = (hp ? Q1 : Q0) - sl * RPL;
#pragma unroll
    for (int k = 0; k < RPL; ++k) {
      const uint32_t v = (bestv[k] >> sh) & 0xFFFFu;
      if (k < nrows && v > bv) {
        bv = v;
        bc = ((bestc[k] >> sh) & 0xFFFFu) - 32u;
        br = (uint32_t)(sl * RPL + k + 1);
      }
    }
#pragma unroll
    for (int d = G / 2; d > 0; d >>= 1) {
      uint32_t ov = __shfl_xor_sync(0xffffffffu, bv, d, G);
      uint32_t oc = __shfl_xor_sync(0xffffffffu, bc, d, G);
      uint32_t orr = __shfl_xor_sync(0xffffffffu, br, d, G);
      if (ov > bv || (ov == bv && orr < br)) {
        bv = ov;
        bc = oc;
        br = orr;
      }
    }
    scorem[hp] = bv > B ? (int)((bv - B) >> 4) : 0;
    cellm[hp] = scorem[hp] > 0 ? (int32_t)(br * (uint32_t)((hp ? R1 : R0) + 1) + bc) : 0;
  }
  if (sl < 2 && (sl == 0 ? has0 : has1)) {
    const int32_t p = sl == 0 ? p0 : p1;
    a.best[p] = make_int2(scorem[sl], cellm[sl]);
  }
}

// One work item of kPairs pairs per warp.
template <int G, int RPL, bool TRACE, bool VAR>
__global__ void __launch_bounds__(kPkWarps * 32, (TRACE || RPL > 13) ? 16 / kPkWarps : 24 / kPkWarps)
    sw_packed_kernel(FastArgs a) {
  constexpr int kPairs = 2 * (32 / G);
  extern __shared__ uint32_t wsel_all[];  // [warps * groups][R + 1]
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t nlist = *a.count - a.list_offset;
  const int64_t warp = (int64_t)blockIdx.x * kPkWarps + wib;
  if (warp * kPairs < nlist) packed_item<G, RPL, TRACE, VAR>(a, warp, nlist, wsel_all, wib, lane);
}

// Traceback walk (src/smithWaterman.cu:911-1026), one thread per printed
// pair: dependent loads of the 4-bit directions the trace pass streamed out;
// many walks in flight hide each other's latency.
constexpr int kWalkThreads = 128;  // small blocks: walks of uneven length leave SMs sooner

template <int G, int RPL>
__global__ void __launch_bounds__(kWalkThreads) sw_walk_kernel(FastArgs a) {
  constexpr int kGroups = 32 / G;
  constexpr int kPairs = 2 * kGroups;
  constexpr int kNW = DirLayout<RPL>::kWords;
  const int64_t nlist = *a.count - a.list_offset;
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nlist || idx >= a.chunk) return;
  const int32_t p = a.list[a.list_offset + idx];
  const int64_t warp = idx / kPairs;
  const int g = (int)((idx % kPairs) >> 1);
  const int hp = (int)(idx & 1);
  const int R = a.R;
  const int S8 = steps8(R, G);
  const uint32_t* dirs = a.dirs + (warp * kGroups + g) * (int64_t)G * kNW * S8;
  const char* qg = a.q + (int64_t)p * a.q_stride;
  const char* wg = a.w + (int64_t)p * a.w_stride;
  const int W = (a.r_len ? a.r_len[p] : R) + 1;  // the pair's own window for cell indices
  const int shift_half = 16 * hp;
  // The walk moves to lower addresses one step (kNW words) per diagonal
  // move inside a lane's rows: the direction words are kept as three
  // 16-byte blocks in registers, the one holding the cell's word and the two
  // before it, so one round of loads serves several steps instead of one
  // dependent load per step.  (The group's region starts 16-byte aligned and
  // holds at least 16 blocks; blocks below its start are never read.)
  const uint4* dirs4 = reinterpret_cast<const uint4*>(dirs);
  int64_t blk = -16;  // first cached block
  uint4 c0 = make_uint4(0, 0, 0, 0), c1 = c0, c2 = c0;
  auto pick = [](const uint4& v, int w) -> uint32_t {
    return w == 0 ? v.x : w == 1 ? v.y : w == 2 ? v.z : v.w;
  };
  // the 2-bit code (2 UP, 1 LEFT, 0 DIAG or NONE) of the cell in row
  // ln * RPL + k + 1 (lane ln, its row k) and column jj: word
  // (ln * S8 + jj + ln - 1) * kNW + k / 8 of the lane streams
  auto code_at = [&](int ln, int k, int jj) -> uint32_t {
    const int64_t at = ((int64_t)ln * S8 + (jj + ln - 1)) * kNW + (k >> 3);
    const int64_t b = at >> 2;
    if (b < blk || b > blk + 2) {
      blk = b >= 2 ? b - 2 : 0;
      c0 = __ldg(dirs4 + blk);
      c1 = __ldg(dirs4 + blk + 1);
      c2 = __ldg(dirs4 + blk + 2);
    }
    const int o = (int)(b - blk), w = (int)(at & 3);
    const uint32_t word = o == 0 ? pick(c0, w) : o == 1 ? pick(c1, w) : pick(c2, w);
    const int rows_w = min(8, RPL - (k & ~7));  // rows of the word, the last lowest
    return (word >> (shift_half + 2 * (rows_w - 1 - (k & 7)))) & 3u;
  };
  // query and window bytes in 16-byte blocks too (rows start 16-byte
  // aligned, strides are multiples of 16)
  const bool blocks16 = ((a.q_stride | a.w_stride) & 15) == 0;
  int qb = -1, wb = -1;
  uint4 q16 = make_uint4(0, 0, 0, 0), w16 = q16;
  auto byte_of = [&](const uint4& v, int o) -> char {
    return (char)((pick(v, o >> 2) >> (8 * (o & 3))) & 0xFFu);
  };
  auto qbyte = [&](int i) -> char {
    if (!blocks16) return qg[i];
    if ((i >> 4) != qb) {
      qb = i >> 4;
      q16 = __ldg(reinterpret_cast<const uint4*>(qg) + qb);
    }
    return byte_of(q16, i & 15);
  };
  auto wbyte = [&](int i) -> char {
    if (!blocks16) return wg[i];
    if ((i >> 4) != wb) {
      wb = i >> 4;
      w16 = __ldg(reinterpret_cast<const uint4*>(wg) + wb);
    }
    return byte_of(w16, i & 15);
  };
  // consensus bytes are gathered four at a time and stored as words
  // (consensus strings are optional: coordinates only when qcons is null)
  const bool cons = a.qcons != nullptr;
  uint32_t* qcw = cons ? reinterpret_cast<uint32_t*>(a.qcons + (int64_t)p * a.cons_stride) : nullptr;
  uint32_t* rcw = cons ? reinterpret_cast<uint32_t*>(a.rcons + (int64_t)p * a.cons_stride) : nullptr;
  uint32_t qacc = 0, racc = 0;
  // Directions of the reference's kernel (NONE, DIAG, UP, LEFT) from the
  // 2-bit codes and the cell's score h, which the walk carries: a cell
  // with code 0 is NONE exactly when h = 0 (any other cell has h > 0).
  enum : int { kNone = 0, kDiag = 1, kUp = 2, kLeft = 3 };
  auto dir_of = [](uint32_t code, int h) -> int {
    return code == 2u ? kUp : code == 1u ? kLeft : (h == 0 ? kNone : kDiag);
  };
  const int m = a.match, x = a.mismatch, o = a.gap_open, e = a.gap_ext;
  auto upc = [](char c) -> char { return (unsigned)(c - 'a') < 26u ? (char)(c - 32) : c; };
  const int2 b = a.best[p];
  int cr = b.y / W, cc = b.y % W;  // current cell
  int h = b.x;                     // its score
  // its lane and row in the lane (kept as the walk moves up)
  int ln = cr > 0 ? (cr - 1) / RPL : 0, k = cr > 0 ? (cr - 1) % RPL : 0;
  int d = (cr == 0 || cc == 0) ? kNone : dir_of(code_at(ln, k, cc), h);
  // One move per step: its consensus bytes (a gap where the row or column
  // stays), then, unless it reached row or column 0, the predecessor's
  // score (the substitution score for a DIAG move; for a gap, gap_ext when
  // the predecessor itself moved the same way, else gap_open) and
  // direction.  The walk ends at a NONE cell or at the border.
  int tick = -1, nref = -1, start = 0;
  while (d != kNone) {
    const bool up = d != kLeft, left = d != kUp;  // row / column move
    const char qc = qbyte(cr - 1), rc = wbyte(cc - 1);
    ++tick;
    nref += left ? 1 : 0;
    {
      const int sh = 8 * (tick & 3);
      racc |= (uint32_t)(uint8_t)(left ? rc : '-') << sh;
      qacc |= (uint32_t)(uint8_t)(up ? qc : '-') << sh;
      if ((tick & 3) == 3) {
        if (cons) {
          rcw[tick >> 2] = racc;
          qcw[tick >> 2] = qacc;
        }
        racc = qacc = 0;
      }
    }
    start = cc;
    const int nr = cr - (up ? 1 : 0), nc = cc - (left ? 1 : 0);
    if (nr == 0 || nc == 0) break;
    if (up && --k < 0) {
      k = RPL - 1;
      --ln;
    }
    const uint32_t pc = code_at(ln, k, nc);
    int nh;
    if (d == kDiag) {
      const char uq = upc(qc), ur = upc(rc);
      nh = h - ((uq == ur || uq == 'N' || ur == 'N') ? m : x);
    } else {
      nh = h - ((d == kUp ? pc == 2u : pc == 1u) ? e : o);
    }
    cr = nr;
    cc = nc;
    h = nh;
    d = dir_of(pc, nh);
  }
  if (cons && tick >= 0 && (tick & 3) != 3) {
    rcw[tick >> 2] = racc;
    qcw[tick >> 2] = qacc;
  }
  DevAln out;
  out.score = b.x;
  out.start = start;
  out.end = start + nref;
  out.len = tick + 1;
  a.aln[p] = out;
}

}  // namespace
}  // namespace swift
