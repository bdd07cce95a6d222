// The NN-descent join's pair distances on the tensor cores (tcgen05), an opt-in build form
// (efg_set_build_precision).  The join (InitIndex::join, base_index.hpp:328-371) needs, for node i
// with new list N (nn ids) and old list O (no ids), the distance of every pair new[p] x new[p+1..]
// and new[p] x old.  With R = N followed by O, all of them are entries above the diagonal of the
// Gram matrix R[0:nn] R^T.  Several nodes share one MMA tile: their new rows first (the tile's
// first rows, at most 128: the MMA's M side), then their old rows (at most TR rows in all: N), so
// that each node's Gram block sits on the diagonal of the tile's R_new R^T; K runs over 64-value
// blocks of a BF16 copy of the base.
//
//   * Three launches per join.  Tiles of TR = 128 rows (128 TMEM columns, three CTAs per SM) take
//     the nodes in order, 32 consecutive nodes at a time from a counter, packed in order; a node
//     with more rows goes to a list that tiles of TR = 256 rows (two CTAs per SM) pack next; a node
//     with more than 128 new entries or 256 rows goes to a second list, scored tile by tile: a
//     block of new entries (the tile's first rows) with a chunk of the candidates after the block,
//     the block's first chunk also covering the pairs within the block.  Each row's pairs in a
//     tile are consecutive slots of its node's pair array.
//   * CTAs are persistent.  Warps 0 and 2-9 gather a tile's rows with 16-byte cp.async copies
//     (eight threads per 128-byte row segment) into a ring of stages in the 128-byte-swizzle
//     K-major layout; each thread waits for its copies, fences them for the tensor cores
//     (fence.proxy.async) and arrives on the stage's barrier.  The same stage is both MMA operands.
//     One thread of warp 1 issues the MMAs into TMEM.  Warps 2-9 copy the Gram rows of 32 new
//     entries at a time out of TMEM (the two warps of each TMEM lane quarter taking alternate
//     32-column groups) into shared memory, then walk those entries' pairs in pair-array order, one
//     pair per thread: distance ||x||^2 + ||y||^2 - 2 x.y, then the join's record step -- the same
//     per-pair array, per-target counts and `found` flags as the FP32 join kernel.
//   * When BF16 holds every value of the base, one product per value; with integer values and
//     squared norms below 2^23 (byte data up to 128 dimensions) every sum is exact, so the distances
//     equal the FP32 join's and the graph is identical.  Other data take the hi + lo split
//     (hi.hi + hi.lo + lo.hi, a relative error near 2^-17 of sum |x_k y_k|): distances, and so pools,
//     can then differ from the FP32 join's in the last bits.
//   * Shared memory is sized so that the CTAs an SM can hold never need more than its 512 TMEM
//     columns: a persistent CTA must never wait in tcgen05.alloc for columns another one holds.
//     Every wait is bounded; one that runs out sets the error word and the CTA leaves after its
//     copies and MMAs.
#include <algorithm>

#include "join.cuh"
#include "tcgen05.cuh"

namespace efg {
namespace {

using namespace tc;

constexpr uint32_t JM = 128;          // new entries per tile (MMA M, TMEM lanes)
constexpr uint32_t JKB = 64;          // BF16 values per k-block
constexpr uint32_t JREC = 8;          // record warps
constexpr uint32_t JRT = JREC * 32;   // record threads
constexpr uint32_t JTHREADS = 64 + JRT;
constexpr uint32_t JPROD = JTHREADS - 32;  // row-gathering threads (every warp but the MMA warp)
constexpr uint32_t JCH = 32;          // nodes taken from the counter at a time
constexpr uint32_t NONE = 0xffffffffu;

// What a launch works on.
enum : uint32_t {
  MODE_ORDER = 0,  // every node in order, TR = 128: larger nodes go to the lists
  MODE_LIST = 1,   // the nodes of list `mid` (<= 128 new entries, <= 256 rows), TR = 256
  MODE_BIG = 2,    // the nodes of list `big`, tile by tile, TR = 256
};

struct JoinArgs {
  const __nv_bfloat16 *hi, *lo;  // BF16 rows of W values (lo only read when terms = 3)
  const uint32_t *new_ids, *new_cnt, *old_ids, *old_cnt;
  const uint64_t* pair_off;
  const float* bound;
  const float* xnorm;  // FP32 squared norms of the base rows
  float* pairdist;
  uint32_t* cnt;
  uint8_t* found;
  uint32_t* next_node;  // node counter of the launch
  uint32_t* mid;        // nodes of 129 to 256 rows: mid[0] their count, then their ids
  uint32_t* big;        // nodes larger than a tile: big[0] their count, then their ids
  int* err;
  uint64_t n;
  uint32_t W, cap, P, check_k, kblocks, terms, nstages, mode;
};

// Offset of new entry p's first pair within the node's pairs (nn new, no old entries).
__device__ __forceinline__ uint64_t pair_row(uint32_t nn, uint32_t no, uint32_t p) {
  return p == 0 ? 0 : (uint64_t)p * (nn - 1) - (uint64_t)p * (p - 1) / 2 + (uint64_t)p * no;
}

__device__ __forceinline__ void rec_sync() { asm volatile("bar.sync 1, %0;" ::"r"(JRT) : "memory"); }

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}

template <uint32_t TR>
struct Tile {
  // CTAs per SM: three 128-column accumulators, or two of 256 (of the SM's 512 TMEM columns)
  static constexpr uint32_t CTAS = TR == 128 ? 3 : 2;
  static constexpr uint32_t PART = TR * 128;  // one k-block of TR rows
  static constexpr uint32_t DLD = TR + 1;     // row stride of the Gram rows in shared memory
  static constexpr uint32_t BLOCK = TR / 2;   // new entries per block of a node larger than a tile
  static size_t smem(uint32_t terms) {
    const uint32_t nstages = terms == 1 ? 2 : 1;
    return 1024 + (size_t)nstages * (terms == 1 ? 1 : 2) * PART + 32 * DLD * 4;
  }
};

template <uint32_t TR>
__global__ void __launch_bounds__(JTHREADS, Tile<TR>::CTAS) tc_join_kernel(const JoinArgs a) {
  using TL = Tile<TR>;
  constexpr uint32_t PART = TL::PART, DLD = TL::DLD;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bar_full[2], bar_empty[2], bar_mma, bar_drain;
  __shared__ uint64_t po_ch[JCH];                  // pair-array offset of each node of the chunk
  __shared__ uint64_t rstart[JM];                  // slot of each tile new entry's first pair
  __shared__ uint32_t id_ch[JCH], nn_ch[JCH], no_ch[JCH];  // the chunk's nodes (nn 0: no pairs here)
  __shared__ uint32_t tslot[JCH], tnb[JCH], tob[JCH];  // tile nodes: chunk slot, first new row, first old row
  __shared__ uint32_t cum[JM + 1];                 // pairs of the tile's new entries before each one
  __shared__ uint8_t rnode[JM];                    // tile node of each new entry
  __shared__ uint32_t rows_sh[TR];                 // the tile's rows: all new entries, then all old ones
  __shared__ float norm_sh[TR];
  __shared__ uint32_t tmem_base_sh, chn_sh, chpos_sh, tn_sh, nsum_sh, tsum_sh;
  __shared__ uint32_t next_k0_sh, next_cn_sh;  // the chunk being fetched (published after a barrier)
  __shared__ int abort_sh, rec_fail_sh, bad_sh;
  // MODE_BIG: the node (id, list lengths, pair offset), the next tile's block of new entries and
  // candidate chunk start, whether it is the block's first (the one with the triangle), the tile
  __shared__ uint32_t bm_node, bm_nn, bm_no, bm_a0, bm_c0, bm_first, bm_tri, bm_tc0, bm_ch;
  __shared__ uint64_t bm_po;
  const uint32_t raw = smem_addr(smem_raw);
  const uint32_t pad = ((raw + 1023u) & ~1023u) - raw;
  const uint32_t sbase = raw + pad;
  const uint32_t stage_bytes = (a.terms == 1 ? 1u : 2u) * PART;
  float* gram = reinterpret_cast<float*>(smem_raw + pad + a.nstages * stage_bytes);  // 32 x DLD
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (uint32_t s = 0; s < a.nstages; ++s) {
      mbar_init(smem_addr(&bar_full[s]), JPROD);
      mbar_init(smem_addr(&bar_empty[s]), 1);
    }
    mbar_init(smem_addr(&bar_mma), 1);
    mbar_init(smem_addr(&bar_drain), 1);
    abort_sh = 0;
    chn_sh = 0;
    chpos_sh = 0;
    bm_node = NONE;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_base_sh)),
                 "r"(TR)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base_sh;
  volatile int* abort_flag = &abort_sh;
  bool mma_issued = false;
  uint64_t kb_done = 0;  // k-blocks of the tiles before this one (position in the stage ring)
  uint32_t tiles = 0;    // tiles multiplied so far (parity of bar_mma)

  for (;;) {
    __syncthreads();  // the previous tile's rows and entry arrays are no longer read
    if (a.mode == MODE_BIG) {
      // ---------------------------------------------------------- the next tile of a listed node
      if (threadIdx.x == 0) {
        uint32_t tn = 0;
        bad_sh = 0;
        rec_fail_sh = 0;
        while (!*abort_flag) {
          if (bm_node == NONE) {
            const uint32_t k = atomicAdd(a.next_node, 1u);
            if (k >= a.big[0]) break;
            const uint32_t i = a.big[1 + k];
            bm_node = i;
            bm_nn = a.new_cnt[i];
            bm_no = a.old_cnt[i];
            bm_po = a.pair_off[i];
            bm_a0 = 0;
            bm_c0 = min(TL::BLOCK, bm_nn);
            bm_first = 1;
          }
          const uint32_t nn = bm_nn, T = nn + bm_no, A = min(TL::BLOCK, nn - bm_a0);
          if (bm_c0 < T || (bm_first && A > 1)) {  // a tile with pairs
            const uint32_t ch = min(TR - A, T - bm_c0);
            bm_tri = bm_first;
            bm_tc0 = bm_c0;
            bm_ch = ch;
            bm_c0 += ch;
            bm_first = 0;
            nsum_sh = A;
            tsum_sh = A + ch;
            tn = 1;
            break;
          }
          bm_a0 += A;  // the next block of new entries, or the next node
          if (bm_a0 >= nn) bm_node = NONE;
          else {
            bm_c0 = min(bm_a0 + TL::BLOCK, nn);
            bm_first = 1;
          }
        }
        tn_sh = tn;
      }
      __syncthreads();
      if (tn_sh == 0) break;
      const uint32_t A = nsum_sh, nn = bm_nn, no = bm_no, a0 = bm_a0, c0 = bm_tc0, tri = bm_tri;
      const uint64_t i = bm_node;
      for (uint32_t b = threadIdx.x; b < tsum_sh; b += JTHREADS) {
        const uint32_t c = b < A ? a0 + b : c0 + (b - A);  // entry of the node's lists (new, then old)
        uint32_t r = c < nn ? a.new_ids[i * a.cap + c] : a.old_ids[i * a.cap + c - nn];
        if (r >= a.n) {  // not a row: reported, the tile left out
          bad_sh = 1;
          r = 0;
        }
        rows_sh[b] = r;
        norm_sh[b] = a.xnorm[r];
        if (b < A) {
          const uint32_t pe = a0 + b;
          rnode[b] = 0;
          rstart[b] = bm_po + pair_row(nn, no, pe) + (tri ? 0 : c0 - pe - 1);
        }
      }
    } else {
      // ---------------------------------------------------------- packed tiles
      // every thread reads the chunk position before thread 0 changes it (below, or in the packing
      // step): a warp that read it late would take another branch and miss the barriers
      const bool fetch = chpos_sh >= chn_sh;
      __syncthreads();
      if (fetch) {  // the chunk is packed: the next JCH nodes
        if (threadIdx.x == 0) {
          const uint32_t total = a.mode == MODE_LIST ? a.mid[0] : (uint32_t)a.n;
          const uint32_t k0 = *abort_flag ? total : atomicAdd(a.next_node, JCH);
          next_cn_sh = k0 < total ? min(JCH, total - k0) : 0;
          next_k0_sh = k0;
        }
        __syncthreads();
        const uint32_t cn = next_cn_sh;
        if (cn == 0) break;
        if (threadIdx.x < cn) {
          const uint32_t k = next_k0_sh + threadIdx.x;
          const uint32_t i = a.mode == MODE_LIST ? a.mid[1 + k] : k;
          uint32_t nn = a.new_cnt[i];
          const uint32_t no = a.old_cnt[i];
          if (nn > a.cap || no > a.cap) {  // not a list: reported, the node left out
            atomicOr(a.err, 4);
            nn = 0;
          } else if (nn > 0 && a.mode == MODE_ORDER && (nn > JM || nn + no > TR)) {
            if (nn <= JM && nn + no <= 256) a.mid[1 + atomicAdd(a.mid, 1u)] = i;  // for TR = 256
            else a.big[1 + atomicAdd(a.big, 1u)] = i;                                // tile by tile
            nn = 0;
          }
          id_ch[threadIdx.x] = i;
          nn_ch[threadIdx.x] = nn;
          no_ch[threadIdx.x] = no;
          po_ch[threadIdx.x] = a.pair_off[i];
        }
        __syncthreads();
        if (threadIdx.x == 0) {
          chn_sh = cn;
          chpos_sh = 0;
        }
      }
      if (threadIdx.x == 0) {  // the next nodes of the chunk that fit one tile together
        const uint32_t cn = chn_sh;
        uint32_t pos = chpos_sh, tn = 0, ns = 0, ts = 0;
        if (*abort_flag) pos = cn;
        while (pos < cn) {
          const uint32_t nn = nn_ch[pos], t = nn + no_ch[pos];
          if (nn == 0) {
            ++pos;
            continue;
          }
          if (ns + nn > JM || ts + t > TR) break;
          tslot[tn] = pos;
          tnb[tn] = ns;
          ns += nn;
          ts += t;
          ++tn;
          ++pos;
        }
        for (uint32_t j = 0, o = ns; j < tn; ++j) {
          tob[j] = o;
          o += no_ch[tslot[j]];
        }
        chpos_sh = pos;
        tn_sh = tn;
        nsum_sh = ns;
        tsum_sh = ts;
        bad_sh = 0;
        rec_fail_sh = 0;
      }
      __syncthreads();
      if (tn_sh == 0) continue;
      for (uint32_t j = warp; j < tn_sh; j += JTHREADS / 32) {  // a warp per tile node
        const uint32_t sl = tslot[j], nn = nn_ch[sl], no = no_ch[sl];
        const uint64_t i = id_ch[sl];
        for (uint32_t e = lane; e < nn + no; e += 32) {
          uint32_t r = e < nn ? a.new_ids[i * a.cap + e] : a.old_ids[i * a.cap + e - nn];
          if (r >= a.n) {  // not a row: reported, the tile left out
            bad_sh = 1;
            r = 0;
          }
          const uint32_t b = e < nn ? tnb[j] + e : tob[j] + e - nn;
          rows_sh[b] = r;
          norm_sh[b] = a.xnorm[r];
          if (e < nn) {
            rnode[b] = (uint8_t)j;
            rstart[b] = po_ch[sl] + pair_row(nn, no, e);
          }
        }
      }
    }
    __syncthreads();
    const uint32_t Ns = nsum_sh, Ts = tsum_sh, Tpad = (Ts + 15) & ~15u;
    if (bad_sh) {
      if (threadIdx.x == 0) atomicOr(a.err, 4);
      continue;
    }

    if (warp != 1) {
      // ------------------------------------------------------------ row gathers (warps 0, 2-9)
      const uint32_t pt = warp == 0 ? lane : threadIdx.x - 32;  // producer index, 0 .. JPROD - 1
      uint32_t s_prev = 0;
      bool ok = true;
      for (uint32_t kb = 0; kb < a.kblocks; ++kb) {
        const uint64_t g = kb_done + kb;
        const uint32_t s = (uint32_t)(g % a.nstages), ph = (uint32_t)((g / a.nstages) & 1);
        if (!mbar_wait(smem_addr(&bar_empty[s]), ph ^ 1u, abort_flag, a.err)) {
          ok = false;
          break;
        }
        const uint32_t st = sbase + s * stage_bytes;
        for (uint32_t e = pt; e < Ts * 8; e += JPROD) {
          const uint32_t r = e >> 3, j = e & 7;
          const uint64_t off = (uint64_t)rows_sh[r] * a.W + kb * JKB + j * 8;
          const uint32_t dst = st + r * 128 + ((j ^ (r & 7)) << 4);
          cp_async16(dst, a.hi + off);
          if (a.terms != 1) cp_async16(dst + PART, a.lo + off);
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
        if (a.nstages > 1 && kb > 0) {  // the previous k-block's copies are done: hand its stage over
          asm volatile("cp.async.wait_group 1;" ::: "memory");
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          mbar_arrive(smem_addr(&bar_full[s_prev]));
        } else if (a.nstages == 1) {
          asm volatile("cp.async.wait_group 0;" ::: "memory");
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          mbar_arrive(smem_addr(&bar_full[s]));
        }
        s_prev = s;
      }
      asm volatile("cp.async.wait_group 0;" ::: "memory");
      if (ok && a.nstages > 1) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_arrive(smem_addr(&bar_full[s_prev]));
      }
    }
    if (warp == 1) {
      // ------------------------------------------------------------ MMAs (one thread)
      if (lane == 0) {
        const uint32_t idesc = idesc_bf16(JM, Tpad);
        bool ok = true;
        for (uint32_t kb = 0; kb < a.kblocks; ++kb) {
          const uint64_t g = kb_done + kb;
          const uint32_t s = (uint32_t)(g % a.nstages), ph = (uint32_t)((g / a.nstages) & 1);
          if (!mbar_wait(smem_addr(&bar_full[s]), ph, abort_flag, a.err)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t st = sbase + s * stage_bytes;
          const uint64_t dh = sw128_desc(st), dl = sw128_desc(st + PART);
#pragma unroll
          for (uint32_t j = 0; j < JKB / 16; ++j) {
            const uint64_t o = (uint64_t)(2 * j);
            umma_bf16(tmem, dh + o, dh + o, idesc, (kb | j) != 0 ? 1u : 0u);
            if (a.terms != 1) {
              umma_bf16(tmem, dh + o, dl + o, idesc, 1u);
              umma_bf16(tmem, dl + o, dh + o, idesc, 1u);
            }
          }
          mma_issued = true;
          umma_commit(smem_addr(&bar_empty[s]));  // the stage is free once these MMAs have read it
        }
        if (ok) umma_commit(smem_addr(&bar_mma));  // the tile's Gram matrix is complete
      }
      __syncwarp();
    } else if (warp >= 2) {
      // ------------------------------------------------------------ records (warps 2-9)
      const uint32_t t = threadIdx.x - 64, quad = warp & 3u, half = (warp - 2) >> 2;
      const bool big = a.mode == MODE_BIG;
      if (warp == 2) {  // cum: prefix sums of the new entries' pair counts
        uint32_t carry = 0;
        for (uint32_t r0 = 0; r0 < Ns; r0 += 32) {
          const uint32_t r = r0 + lane;
          uint32_t v = 0;
          if (r < Ns) {
            if (big) {
              v = (bm_tri ? Ns - r - 1 : 0) + bm_ch;
            } else {
              const uint32_t j = rnode[r], sl = tslot[j];
              v = nn_ch[sl] + no_ch[sl] - 1 - (r - tnb[j]);
            }
          }
#pragma unroll
          for (uint32_t o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += u;
          }
          if (r < Ns) cum[r + 1] = carry + v;
          carry += __shfl_sync(0xffffffffu, v, 31);
        }
        if (lane == 0) cum[0] = 0;
      }
      if (!__all_sync(0xffffffffu, mbar_wait(smem_addr(&bar_mma), tiles & 1u, abort_flag, a.err)) && lane == 0)
        rec_fail_sh = 1;
      rec_sync();
      if (!rec_fail_sh) {  // the same for every record warp (written only before the barrier)
        tc_fence_after();
        for (uint32_t q0 = 0; q0 < Ns; q0 += 32) {
          if (quad == q0 / 32) {  // the two warps that can read TMEM lanes q0 .. q0 + 31
            for (uint32_t c0 = half * 32; c0 < Tpad; c0 += 64) {
              uint32_t v[32];
              const uint32_t taddr = tmem + (q0 << 16) + c0;
              tmem_ld16(taddr, v);
              if (c0 + 16 < Tpad) tmem_ld16(taddr + 16, v + 16);
              tmem_wait();
              float* row = gram + lane * DLD + c0;
#pragma unroll
              for (uint32_t j = 0; j < 32; ++j)
                if (c0 + j < Tpad) row[j] = __uint_as_float(v[j]);
            }
          }
          rec_sync();
          // pairs of new entries q0 .. q1 - 1 (in order of entry, then candidate), one per thread
          const uint32_t q1 = min(Ns, q0 + 32), u1 = cum[q1];
          uint32_t r = q0;
          for (uint32_t u = cum[q0] + t; u < u1; u += JRT) {
            while (u >= cum[r + 1]) ++r;
            const uint32_t off = u - cum[r];
            uint32_t bc;    // the candidate's row in the tile
            bool cand_new;  // the candidate is a new entry
            uint64_t node;
            if (big) {
              const uint32_t tl = bm_tri ? Ns - r - 1 : 0;  // the row's pairs within the new block
              if (off < tl) {
                bc = r + 1 + off;
                cand_new = true;
              } else {
                bc = Ns + (off - tl);
                cand_new = bm_tc0 + (off - tl) < bm_nn;
              }
              node = bm_node;
            } else {
              const uint32_t j = rnode[r], sl = tslot[j], nn = nn_ch[sl];
              const uint32_t cl = r - tnb[j] + 1 + off;  // candidate within the node's lists
              bc = cl < nn ? tnb[j] + cl : tob[j] + (cl - nn);
              cand_new = cl < nn;
              node = id_ch[sl];
            }
            const float dot = gram[(r - q0) * DLD + bc];
            const float d = fmaxf(fmaf(-2.f, dot, norm_sh[r] + norm_sh[bc]), 0.f);
            if (join_lane_record<0>(node, rows_sh[r], rows_sh[bc], cand_new, d, rstart[r] + off, a.P, a.check_k,
                                    a.bound, a.pairdist, a.cnt, nullptr, nullptr, nullptr, nullptr))
              a.found[node] = 1;
          }
          rec_sync();  // the Gram rows are overwritten by the next 32 entries
        }
      }
      tc_fence_before();
    }
    kb_done += a.kblocks;
    ++tiles;
  }

  // ------------------------------------------------------------------------------ teardown
  asm volatile("cp.async.wait_all;" ::: "memory");  // no copy of this thread is still in flight
  __syncthreads();
  if (warp == 1) {
    if (lane == 0 && mma_issued) {  // the MMAs have finished before TMEM is freed
      umma_commit(smem_addr(&bar_drain));
      const unsigned long long t0 = clock64();
      while (!mbar_try_wait(smem_addr(&bar_drain), 0)) {
        if (clock64() - t0 > WAIT_CYCLES) {
          atomicOr(a.err, 2);
          break;
        }
      }
    }
    __syncwarp();
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TR) : "memory");
  }
}

// One launch of tc_join_kernel<TR>: persistent CTAs, Tile<TR>::CTAS per SM.
template <uint32_t TR>
int launch_join(const JoinArgs& a, int sms, int smem_max, cudaStream_t s) {
  // shared memory keeps the CTAs of an SM within its TMEM columns: more than CTAS of them must not
  // fit
  size_t smem = Tile<TR>::smem(a.terms);
  int dev = 0, sm_smem = 0, reserved = 0;
  EFG_CUDA(cudaGetDevice(&dev));
  EFG_CUDA(cudaDeviceGetAttribute(&sm_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
  EFG_CUDA(cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev));
  cudaFuncAttributes fa;
  EFG_CUDA(cudaFuncGetAttributes(&fa, tc_join_kernel<TR>));
  const size_t fixed = fa.sharedSizeBytes + (size_t)reserved;
  const size_t floor_per_cta = (size_t)sm_smem / (Tile<TR>::CTAS + 1) + 1;  // more than CTAS do not fit
  if (smem + fixed < floor_per_cta) smem = floor_per_cta - fixed;
  if ((int64_t)smem > smem_max) return fail(EFG_ERR_ARG, "tensor-core join: shared memory");
  EFG_CUDA(cudaFuncSetAttribute(tc_join_kernel<TR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  EFG_CUDA(cudaFuncSetAttribute(tc_join_kernel<TR>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                (int)cudaSharedmemCarveoutMaxShared));
  // (the occupancy calculator can answer fewer CTAs than fit; the CTAs are persistent, so one that
  // does not fit beside the others starts after them and finds the node counter spent)
  tc_join_kernel<TR><<<(unsigned)(sms * Tile<TR>::CTAS), JTHREADS, smem, s>>>(a);
  EFG_CUDA(cudaGetLastError());
  return EFG_OK;
}

}  // namespace

// The BF16 rows (hi, and lo = x - hi), FP32 squared norms and the inexact flag (some lo not zero)
// of the base, for the tensor-core join: rows of W = round_up(dim, 64) values.
int tc_join_prepare(const float* base, uint64_t n, uint32_t dim, uint32_t ld, __nv_bfloat16* hi, __nv_bfloat16* lo,
                    float* norms, int* inexact, cudaStream_t s) {
  const uint32_t W = (dim + 63) / 64 * 64;
  int dev = 0, sms = 148;
  EFG_CUDA(cudaGetDevice(&dev));
  EFG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  EFG_CUDA(cudaMemsetAsync(inexact, 0, sizeof(int), s));
  const uint64_t warps = std::max<uint64_t>(1, std::min<uint64_t>(n, (uint64_t)sms * 64));
  to_bf16_kernel<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, s>>>(base, n, dim, ld, W, hi, lo, norms, n, inexact);
  EFG_CUDA(cudaGetLastError());
  return EFG_OK;
}

// Join pass 0 on the tensor cores: three launches (tiles of 128 rows over every node, tiles of 256
// rows over the nodes listed in mid, and the nodes listed in big tile by tile).  counters: three
// node counters, zero on entry; mid and big: n + 1 words each, their counts (word 0) zero on entry;
// *err zero on entry.  terms: 1 (BF16 holds the base) or 3 (hi + lo products).
int tc_join(const __nv_bfloat16* hi, const __nv_bfloat16* lo, const float* norms, uint64_t n, uint32_t dim,
            uint32_t terms, uint32_t cap, uint32_t P, uint32_t check_k, const uint32_t* new_ids,
            const uint32_t* new_cnt, const uint32_t* old_ids, const uint32_t* old_cnt, const uint64_t* pair_off,
            const float* bound, float* pairdist, uint32_t* cnt, uint8_t* found, uint32_t* counters, uint32_t* mid,
            uint32_t* big, int* err, cudaStream_t s) {
  if (terms != 1 && terms != 3) return fail(EFG_ERR_ARG, "tensor-core join: terms must be 1 or 3");
  if (n >= 0xffffffffull) return fail(EFG_ERR_ARG, "tensor-core join: more than 2^32 - 2 rows");
  const uint32_t W = (dim + 63) / 64 * 64;
  int dev = 0, sms = 148, smem_max = 0;
  EFG_CUDA(cudaGetDevice(&dev));
  EFG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  EFG_CUDA(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  JoinArgs a;
  a.hi = hi;
  a.lo = terms == 1 ? hi : lo;
  a.new_ids = new_ids;
  a.new_cnt = new_cnt;
  a.old_ids = old_ids;
  a.old_cnt = old_cnt;
  a.pair_off = pair_off;
  a.bound = bound;
  a.xnorm = norms;
  a.pairdist = pairdist;
  a.cnt = cnt;
  a.found = found;
  a.mid = mid;
  a.big = big;
  a.err = err;
  a.n = n;
  a.W = W;
  a.cap = cap;
  a.P = P;
  a.check_k = check_k;
  a.kblocks = W / JKB;
  a.terms = terms;
  a.nstages = terms == 1 ? 2 : 1;
  a.mode = MODE_ORDER;
  a.next_node = counters;
  EFG_TRY(launch_join<128>(a, sms, smem_max, s));
  a.mode = MODE_LIST;
  a.next_node = counters + 1;
  EFG_TRY(launch_join<256>(a, sms, smem_max, s));
  a.mode = MODE_BIG;
  a.next_node = counters + 2;
  EFG_TRY(launch_join<256>(a, sms, smem_max, s));
  return EFG_OK;
}

}  // namespace efg
