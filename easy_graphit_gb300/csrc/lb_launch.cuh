// Kernels wrapping the load-balancing device functions, and the host-side
// dispatch of one edgeset.apply launch (the switch of operators.cpp:631-647).
// Included by one translation unit per UDF so each UDF's kernels compile in
// parallel.
#pragma once

#include "engine.h"
#include "lb.cuh"
#include "udf.cuh"

namespace gg {

template <class F>
__global__ void __launch_bounds__(1024) k_vertex(DGraph g, Enum en, F f, DOut out) {
  const int32_t n = en.count();
  const int32_t nv = ceil_div(n, blockDim.x);
  for (int32_t v = blockIdx.x; v < nv; v += gridDim.x) lb_vertex(g, en, n, f, out, v);
}

template <class F>
__global__ void __launch_bounds__(1024) k_wm(DGraph g, Enum en, F f, DOut out) {
  const int32_t n = en.count();
  const int32_t nv = ceil_div(n, blockDim.x >> 5);
  for (int32_t v = blockIdx.x; v < nv; v += gridDim.x) lb_wm(g, en, n, f, out, v);
}

// One whole CTA per enumerated vertex (TWC large bin).
template <class F>
__global__ void __launch_bounds__(1024) k_cta(DGraph g, Enum en, F f, DOut out) {
  const int32_t n = en.count();
  for (int32_t v = blockIdx.x; v < n; v += gridDim.x) {
    const int32_t s = en.at(v);
    do_range(g, f, out, s, __ldg(g.off + s), __ldg(g.off + s + 1), threadIdx.x, blockDim.x);
  }
}

template <class F, bool kCtaBin>
__global__ void __launch_bounds__(1024)
    k_twce(DGraph g, Enum en, F f, DOut out, int32_t *chunks, int32_t *chunk_cnt, int32_t chunk) {
  extern __shared__ int4 smem_raw[];
  TwceSmem &sm = *reinterpret_cast<TwceSmem *>(smem_raw);
  const int32_t n = en.count();
  const int32_t nv = ceil_div(n, blockDim.x / kStage1);
  for (int32_t v = blockIdx.x; v < nv; v += gridDim.x)
    lb_twce<F, kCtaBin>(g, en, n, f, out, v, sm, chunks, chunk_cnt, chunk);
}

template <class F>
__global__ void __launch_bounds__(1024)
    k_chunks(DGraph g, const int32_t *chunks, const int32_t *chunk_cnt, F f, DOut out) {
  const int32_t n = *(volatile const int32_t *)chunk_cnt;
  for (int32_t v = blockIdx.x; v < n; v += gridDim.x) lb_chunk(g, chunks, f, out, v);
}

template <class F>
__global__ void __launch_bounds__(1024) k_cm(DGraph g, Enum en, F f, DOut out) {
  extern __shared__ int4 smem_raw[];
  CmSmem &sm = *reinterpret_cast<CmSmem *>(smem_raw);
  const int32_t n = en.count();
  const int32_t nv = ceil_div(n, blockDim.x);
  for (int32_t v = blockIdx.x; v < nv; v += gridDim.x) lb_cm(g, en, n, f, out, v, sm);
}

template <class F>
__global__ void __launch_bounds__(1024)
    k_strict(DGraph g, Enum en, const int32_t *sum, F f, DOut out, int32_t per) {
  const int32_t n = en.count();
  const int32_t nv = ceil_div(sum[n], per);
  for (int32_t v = blockIdx.x; v < nv; v += gridDim.x) lb_strict(g, en, n, sum, f, out, v, per);
}

template <class F>
__global__ void __launch_bounds__(1024) k_edge_only(DGraph g, F f, DOut out) {
  lb_edge_only(g, f, out, (int64_t)blockIdx.x * blockDim.x + threadIdx.x,
               (int64_t)gridDim.x * blockDim.x);
}

template <class F>
__global__ void __launch_bounds__(1024) k_edge_only_blocked(DGraph g, F f, DOut out) {
  lb_edge_only_blocked(g, f, out, (int64_t)blockIdx.x * blockDim.x + threadIdx.x,
                       (int64_t)gridDim.x * blockDim.x);
}

// Helpers implemented in frontier.cu (not UDF-specific).
gg_status twc_bin(gg_graph *G, const DGraph &g, const Enum &en, int32_t n_host, int32_t cta,
                  int32_t **bins, int32_t **bin_cnt);
gg_status strict_scan(gg_graph *G, const DGraph &g, const Enum &en, int32_t n_host,
                      int32_t **sum);
gg_status etwc_scratch(gg_graph *G, int64_t max_chunks, int32_t **chunks, int32_t **cnt);

template <class K>
inline int grid_for(K kernel, int cta, size_t smem, int sm_count, int64_t nvcta) {
  const int res = resident_grid((const void *)kernel, cta, smem, sm_count);
  if (nvcta < 0) return res;
  return (int)std::max<int64_t>(1, std::min<int64_t>(nvcta, res));
}

template <class F>
gg_status launch_lb(const EdgeLaunch &L, const F &f) {
  gg_graph *G = L.graph;
  cudaStream_t st = G->stream;
  const int cta = L.cta;
  const int sms = G->sm_count;
  const int64_t n = L.n_host;
  if (n == 0 && L.lb != GG_LB_EDGE_ONLY) return GG_OK;
  switch (L.lb) {
    case GG_LB_EDGE_ONLY: {
      if (L.g.nbuckets > 0) {
        auto k = k_edge_only_blocked<F>;
        { gg::note_launch(); k<<<grid_for(k, cta, 0, sms, -1), cta, 0, st>>>(L.g, f, L.out); }
      } else {
        auto k = k_edge_only<F>;
        { gg::note_launch(); k<<<grid_for(k, cta, 0, sms, -1), cta, 0, st>>>(L.g, f, L.out); }
      }
      break;
    }
    case GG_LB_VERTEX_BASED: {
      auto k = k_vertex<F>;
      { gg::note_launch(); k<<<grid_for(k, cta, 0, sms, n < 0 ? -1 : ceil_div(n, cta)), cta, 0, st>>>(L.g, L.en, f, L.out); }
      break;
    }
    case GG_LB_WM: {
      auto k = k_wm<F>;
      { gg::note_launch(); k<<<grid_for(k, cta, 0, sms, n < 0 ? -1 : ceil_div(n, cta / 32)), cta, 0, st>>>(L.g, L.en, f,
                                                                                     L.out); }
      break;
    }
    case GG_LB_TWCE: {
      auto k = k_twce<F, true>;
      const size_t sm = twce_smem_bytes(cta);
      { gg::note_launch(); k<<<grid_for(k, cta, sm, sms, n < 0 ? -1 : ceil_div(n, cta / kStage1)), cta, sm, st>>>(
          L.g, L.en, f, L.out, nullptr, nullptr, 0); }
      break;
    }
    case GG_LB_ETWC: {
      // Stage 1+2 in-CTA, hub edges as chunks of 4*cta edges on a global list.
      const int32_t chunk = 4 * cta;
      int32_t *chunks = nullptr, *cnt = nullptr;
      const int64_t maxc = (int64_t)L.g.E / chunk + (n < 0 ? L.g.V : n) + 1;
      GG_TRY(etwc_scratch(G, maxc, &chunks, &cnt));
      GG_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int32_t), st));
      auto k = k_twce<F, false>;
      const size_t sm = twce_smem_bytes(cta);
      { gg::note_launch(); k<<<grid_for(k, cta, sm, sms, n < 0 ? -1 : ceil_div(n, cta / kStage1)), cta, sm, st>>>(
          L.g, L.en, f, L.out, chunks, cnt, chunk); }
      auto k2 = k_chunks<F>;
      { gg::note_launch(); k2<<<grid_for(k2, cta, 0, sms, -1), cta, 0, st>>>(L.g, chunks, cnt, f, L.out); }
      break;
    }
    case GG_LB_CM: {
      auto k = k_cm<F>;
      const size_t sm = cm_smem_bytes(cta);
      { gg::note_launch(); k<<<grid_for(k, cta, sm, sms, n < 0 ? -1 : ceil_div(n, cta)), cta, sm, st>>>(L.g, L.en, f,
                                                                                  L.out); }
      break;
    }
    case GG_LB_TWC: {
      int32_t *bins = nullptr, *bin_cnt = nullptr;
      GG_TRY(twc_bin(G, L.g, L.en, (int32_t)n, cta, &bins, &bin_cnt));
      const int64_t cap = n < 0 ? L.g.V : n;
      Enum small{bins, bin_cnt + 0, -1}, mid{bins + cap, bin_cnt + 1, -1},
          large{bins + 2 * cap, bin_cnt + 2, -1};
      auto k1 = k_vertex<F>;
      auto k2 = k_wm<F>;
      auto k3 = k_cta<F>;
      { gg::note_launch(); k1<<<grid_for(k1, cta, 0, sms, -1), cta, 0, st>>>(L.g, small, f, L.out); }
      { gg::note_launch(); k2<<<grid_for(k2, cta, 0, sms, -1), cta, 0, st>>>(L.g, mid, f, L.out); }
      { gg::note_launch(); k3<<<grid_for(k3, cta, 0, sms, -1), cta, 0, st>>>(L.g, large, f, L.out); }
      break;
    }
    case GG_LB_STRICT: {
      int32_t *sum = nullptr;
      GG_TRY(strict_scan(G, L.g, L.en, (int32_t)n, &sum));
      auto k = k_strict<F>;
      { gg::note_launch(); k<<<grid_for(k, cta, 0, sms, -1), cta, 0, st>>>(L.g, L.en, sum, f, L.out, 8 * cta); }
      break;
    }
    default:
      return set_error(GG_ERR_UNSUPPORTED, "load balancing %d not supported", L.lb);
  }
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

template <class U>
gg_status launch_dir(const EdgeLaunch &L, const U &u) {
  if (L.pull) return launch_lb(L, EdgeF<U, true>{u, L.in_src, L.in_dst, L.filter});
  return launch_lb(L, EdgeF<U, false>{u, L.in_src, L.in_dst, L.filter});
}

}  // namespace gg
