// Two-CTA cluster form of the persistent split-precision contraction.
//
// The two CTAs of a cluster work on the same A tile (same triplet slot, job, x, y-block and term)
// and on adjacent N blocks (nb = 2 nbp + cluster rank), so the A tile - the large operand, re-read
// by every N block - crosses L2 once for both: each CTA loads the digit planes of its parity
// (p % 2 == rank) with a cluster multicast into both CTAs' shared memory, and its own B tile
// without multicast.  This cuts the L2 -> SM bytes per digit-plane product by ~1.5x, the bound of
// the single-CTA kernel once its epilogue keeps up.
//
// Scheduling is static: cluster c takes the pair items c, c + nclusters, ... of the host's
// cost-ordered table, so both CTAs walk the same sequence without exchanging item ids.
// Synchronisation across the pair:
//   full[s]  (count 1, local): the local producer's arrive.expect_tx for the whole stage; the A
//            planes arrive from both CTAs' multicasts, B from the local load;
//   empty[s] (count 2): both CTAs' MMA issuers commit with a cluster multicast, so a producer that
//            sees empty[s] knows stage s is free in both CTAs before it multicasts into it.
// A cluster barrier follows the mbarrier initialisation (no remote arrival or multicast reaches
// an uninitialised barrier) and precedes exit (after each producer has seen the last use of every
// stage consumed by both MMAs, so nothing is still in flight towards this CTA's shared memory).
// Every mbarrier wait is bounded (sm100::kSpinLimit); a CTA that gives up sets the error flag,
// and its peer's waits then give up too, so both reach the final cluster barrier.
#pragma once

#include "oz_persist.cuh"

namespace ccsdt {

struct PzPairItem {
  int slot, job, x, yb, nbp;
};
// pair item id -> fields; ids are dense in (slot, job, x, yb, nbp), nbp fastest
__device__ __forceinline__ PzPairItem pz_decode_pair(unsigned id, int v, int yblocks, int npairs) {
  PzPairItem it;
  it.nbp = id % npairs;
  id /= npairs;
  it.yb = id % yblocks;
  id /= yblocks;
  it.x = id % v;
  id /= v;
  it.job  = id % 3;
  it.slot = id / 3;
  return it;
}

__device__ __forceinline__ int pz_plane_map(int mapA) {
  return mapA == PZ_OVVV_NAT ? PZ_OVVV_NAT_P1 : mapA == PZ_OVVV_SWP ? PZ_OVVV_SWP_P1 : PZ_OOOVH_A_P1;
}

template<int S, int NT, int STAGES, int KC>
__global__ void __launch_bounds__(PZ_THREADS, 1) oz_pair_kernel(const __grid_constant__ PzParams P) {
  using C = PzCfg<S, NT, STAGES, KC>;
  constexpr uint16_t kBoth = 0x3;
  const int      v = P.v, yblocks = (v + PZ_BM - 1) / PZ_BM, nblocks = (v + NT - 1) / NT, npairs = (nblocks + 1) / 2;
  const int      base = P.base ? *P.base : 0;
  const int      rank = (int) sm100::cluster_ctarank();
  const unsigned cid = sm100::cluster_id_x(), ncl = sm100::cluster_count_x();

  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full      = reinterpret_cast<uint64_t*>(smem + STAGES * C::STAGE_BYTES);
  uint64_t* empty     = full + STAGES;
  uint64_t* lvl_full  = empty + STAGES; // [NBUF] MMAs of a term done
  uint64_t* lvl_empty = lvl_full + 3;   // [NBUF] epilogue drained the buffer
  uint64_t* drain     = lvl_empty + 3;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if(threadIdx.x == 0) {
    for(int s = 0; s < STAGES; s++) {
      sm100::mbar_init(&full[s], 1);
      sm100::mbar_init(&empty[s], 2); // one commit from each CTA's MMA issuer
    }
    for(int b = 0; b < C::NBUF; b++) {
      sm100::mbar_init(&lvl_full[b], 1);
      sm100::mbar_init(&lvl_empty[b], PZ_EPI);
    }
    sm100::mbar_init(drain, 1);
    *abort_flag = 0;
    sm100::mbar_fence_init();
  }
  if(warp == 1) {
    sm100::tmem_alloc(tmem_slot, C::TMEM_COLS);
    sm100::tmem_relinquish();
  }
  sm100::tc_fence_before();
  __syncthreads();
  sm100::cluster_sync(); // both CTAs' barriers are initialised before any multicast or remote arrival
  sm100::tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  auto fail = [&]() {
    *abort_flag = 1;
    if(P.err) atomicExch(P.err, 1);
  };
  // this cluster's items: table entries cid, cid + ncl, ...
  const unsigned n_mine = P.nitems > cid ? (P.nitems - cid + ncl - 1) / ncl : 0;
  auto decode = [&](unsigned id) {
    const PzPairItem pi = pz_decode_pair(id, v, yblocks, npairs);
    return PzItem{pi.slot, pi.job, pi.x, pi.yb, 2 * pi.nbp + rank};
  };
  // item ids two ahead and triplet entries one ahead, so the loads of the next item overlap the
  // current one: id(kk) -> entry(kk)
  auto id_at = [&](unsigned kk) { return kk < n_mine ? P.order[cid + kk * ncl] : 0u; };
  auto entry = [&](unsigned id) { return reinterpret_cast<const int4*>(P.tri)[base + decode(id).slot]; };

  if(warp == 0) {
    // ------------------------------------------------------------ TMA producer
    if(lane == 0) {
      for(int m: {PZ_OVVV_NAT_P1, PZ_OVVV_SWP_P1, PZ_T2, PZ_T2H_NAT_B, PZ_T2H_SWP_B, PZ_OOOVH_A_P1})
        sm100::prefetch_tmap(&P.maps[m]);
      int      stage_it = 0;
      bool     ok       = true;
      unsigned id0 = id_at(0), id1 = id_at(1);
      int4     e0  = n_mine ? entry(id0) : make_int4(0, 0, 0, 0);
      for(unsigned kk = 0; ok && !*abort_flag && kk < n_mine; kk++) {
        const PzItem w = decode(id0);
        const int    i = e0.x, j = e0.y, k = e0.z;
        const unsigned id2 = id_at(kk + 2);                        // prefetch
        const int4     e1  = kk + 1 < n_mine ? entry(id1) : e0;
        id0 = id1, id1 = id2;
        for(int t = 0; t < PZ_TERMS && ok; t++) {
          const PzTerm T  = pz_term(P, w.job, t, i, j, k, w.x);
          const int    mA = pz_plane_map(T.mapA);
          for(int k0 = 0; k0 < T.Kp; k0 += KC, stage_it++) {
            const int s = stage_it % STAGES, use = stage_it / STAGES;
            if(use > 0 && !sm100::mbar_wait(&empty[s], (use - 1) & 1)) {
              fail();
              ok = false;
              break;
            }
            unsigned char* a = smem + s * C::STAGE_BYTES;
            sm100::mbar_arrive_expect_tx(&full[s], C::STAGE_BYTES);
#pragma unroll
            for(int p = 0; p < S; p++)
              if((p & 1) == rank)
                sm100::tma_load_5d_mc(a + p * PZ_BM * KC * 2, &P.maps[mA], &full[s], k0, w.yb * PZ_BM, T.a2, T.a3, p, kBoth);
            sm100::tma_load_5d(a + C::A_BYTES, &P.maps[T.mapB], &full[s], k0, w.nb * NT, T.b2, T.b3, 0);
          }
        }
        e0 = e1;
      }
      // the last use of every stage consumed by both MMA issuers: their commits have landed
      // here and no load towards this CTA's shared memory is still in flight
      for(int u = (stage_it > STAGES ? stage_it - STAGES : 0); u < stage_it; u++)
        if(!sm100::mbar_wait(&empty[u % STAGES], (u / STAGES) & 1)) fail();
    }
  } else if(warp == 1) {
    // ------------------------------------------------------------ MMA issuer (the warp runs the
    // loop, lane 0 issues; the gate warp does its waits, see pz_gate_sync).  The MMAs need no item data; between stages the
    // loop does as little as it can (no modulo, no shared-memory reads).
    const uint32_t a0 = sm100::smem_u32(smem);
    uint32_t       a = a0;
    int            s = 0, term_it = 0;
    bool           stop = false;
    for(unsigned kk = 0; !stop && kk < n_mine; kk++) {
      for(int t = 0; t < PZ_TERMS && !stop; t++, term_it++) {
        const int      nst   = (t < 2 ? P.kp_v : P.kp_o) / KC;
        const uint32_t dbase = tmem + (term_it % C::NBUF) * S * NT;
        for(int u = 0; u < nst; u++) {
          if((stop = pz_gate_sync(false))) break;
          sm100::tc_fence_after();
          pz_issue_stage<S, NT, KC>(dbase, a, a + C::A_BYTES, u == 0, lane == 0);
          sm100::mma_commit_mc_if(&empty[s], kBoth, lane == 0); // stage free here, as seen by both producers
          a += C::STAGE_BYTES;
          if(++s == STAGES) s = 0, a = a0;
        }
        if(!stop) sm100::mma_commit_if(&lvl_full[term_it % C::NBUF], lane == 0);
      }
    }
    if(lane == 0) {
      sm100::mma_commit(drain);
      if(!sm100::mbar_wait(drain, 0)) fail();
    }
  } else if(warp == 2) {
    // ------------------------------------------------------------ gate: the MMA issuer's waits
    int  stage_it = 0, term_it = 0;
    bool stop     = false;
    for(unsigned kk = 0; !stop && kk < n_mine; kk++) {
      for(int t = 0; t < PZ_TERMS && !stop; t++, term_it++) {
        const int nst = (t < 2 ? P.kp_v : P.kp_o) / KC;
        const int buf = term_it % C::NBUF;
        int       ok  = 1;
        if(lane == 0 && term_it >= C::NBUF) ok = sm100::mbar_wait(&lvl_empty[buf], ((term_it / C::NBUF) - 1) & 1);
        for(int u = 0; u < nst; u++, stage_it++) {
          bool mine = false;
          if(lane == 0) {
            if(ok) ok = sm100::mbar_wait(&full[stage_it % STAGES], (stage_it / STAGES) & 1);
            if(!ok) fail();
            mine = !ok || *abort_flag;
          }
          __syncwarp();
          if((stop = pz_gate_sync(mine))) break;
        }
      }
    }
  } else {
    // ------------------------------------------------------------ epilogue: PZ_EPI warps
    const int      q = warp & 3, cq = (warp - PZ_EPI_W0) >> 2; // TMEM lane quarter, column quarter
    const int      row = q * 32 + lane;
    const uint32_t lane_base = tmem + ((uint32_t) (q * 32) << 16);
    const int      c_lo = cq * C::COLS;
    int            term_it = 0;
    float          tsq = 0.f;
    int            tail_slot = -1;
    unsigned id0 = id_at(0), id1 = id_at(1);
    int4     e0  = n_mine ? entry(id0) : make_int4(0, 0, 0, 0);
    for(unsigned kk = 0; kk < n_mine; kk++) {
      const PzItem   w   = decode(id0);
      const int      tp[4] = {e0.x, e0.y, e0.z, e0.w};
      const unsigned id2 = id_at(kk + 2);                          // prefetch
      const int4     e1  = kk + 1 < n_mine ? entry(id1) : e0;
      id0 = id1, id1 = id2;
      if(P.tail && tp[3] != tail_slot) {
        if(tail_slot >= 0) pz_flush_tail(P.tail, tail_slot, tsq, lane);
        tsq       = 0.f;
        tail_slot = tp[3];
      }
      if(!pz_epilogue_item<S, NT, C::NBUF>(P, w, w.nb, tp, lane_base, c_lo, row, lane, term_it, tsq, lvl_full, lvl_empty,
                                  abort_flag)) {
        fail();
        break;
      }
      e0 = e1;
    }
    if(P.tail && tail_slot >= 0) pz_flush_tail(P.tail, tail_slot, tsq, lane);
  }
  sm100::tc_fence_before();
  __syncthreads();
  sm100::cluster_sync(); // the peer is done with this CTA's barriers and shared memory
  if(warp == 1) {
    sm100::tc_fence_after();
    sm100::tmem_dealloc(tmem, C::TMEM_COLS);
  }
}

} // namespace ccsdt
