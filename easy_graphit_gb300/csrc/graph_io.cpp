// Host-side graph construction and I/O for libgg.so.
//
// The engine consumes int32 CSR exactly as graphit_runtime::load_graph lays it
// out (runtime/infra_gpu/graph.h:276-294).  The inputs are built the way the
// reference's vendored GAPBS builds them:
//   * R-MAT edge lists: Graph500 bit recursion with per-2^18-edge reseeding of a
//     std::mt19937, followed by a std::shuffle id permutation
//     (infra_gapbs/generator.h:45-55, 74-107), weights U[wmin,wmax] drawn with
//     the same block reseeding (generator.h:125-139);
//   * CSR build + "squish": neighbour lists sorted by (id, weight), duplicates
//     merged keeping the first (= smallest weight), self-loops removed
//     (infra_gapbs/builder.h:73-84, 134-163, 188-226).
// The same std:: engines and distributions are used, so the resulting graphs are
// bit-identical to GAPBS's; oracle/ref_gapbs.cpp checks that against the
// reference's own headers.
#include <algorithm>
#include <atomic>
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <limits>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "gg_internal.h"

namespace {

constexpr int64_t kBlock = int64_t(1) << 18;  // generator.h:145

struct WEdge {
  int32_t u, v, w;
};

// Builds the squished CSR from a weighted edge list.
gg_status build_csr(int64_t num_nodes, const std::vector<WEdge> &el,
                    bool symmetrize, gg_host_graph **out) {
  if (num_nodes <= 0 || num_nodes > std::numeric_limits<int32_t>::max() - 1)
    return gg::set_error(GG_ERR_INVALID, "vertex count %lld out of int32 range",
                         (long long)num_nodes);
  const int64_t V = num_nodes;
  const int64_t M = (int64_t)el.size();
  for (int64_t i = 0; i < M; ++i) {
    if (el[i].u < 0 || el[i].u >= V || el[i].v < 0 || el[i].v >= V)
      return gg::set_error(GG_ERR_INVALID, "edge %lld (%d,%d) out of range",
                           (long long)i, el[i].u, el[i].v);
  }
  // Degree count (both directions when symmetrizing).
  std::vector<int64_t> deg(V + 1, 0);
  {
    std::vector<std::atomic<int64_t>> d(V);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < V; ++i) d[i].store(0, std::memory_order_relaxed);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < M; ++i) {
      d[el[i].u].fetch_add(1, std::memory_order_relaxed);
      if (symmetrize) d[el[i].v].fetch_add(1, std::memory_order_relaxed);
    }
    int64_t run = 0;
    for (int64_t i = 0; i < V; ++i) {
      deg[i] = run;
      run += d[i].load(std::memory_order_relaxed);
    }
    deg[V] = run;
  }
  const int64_t slots = deg[V];
  // Scatter packed (neighbour << 32 | weight) keys; sorting a vertex's keys
  // orders by (id, weight) like NodeWeight::operator< (infra_gapbs/graph.h).
  std::vector<uint64_t> keys(slots);
  {
    std::vector<std::atomic<int64_t>> pos(V);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < V; ++i) pos[i].store(deg[i], std::memory_order_relaxed);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < M; ++i) {
      const WEdge e = el[i];
      keys[pos[e.u].fetch_add(1, std::memory_order_relaxed)] =
          (uint64_t(uint32_t(e.v)) << 32) | uint32_t(e.w);
      if (symmetrize)
        keys[pos[e.v].fetch_add(1, std::memory_order_relaxed)] =
            (uint64_t(uint32_t(e.u)) << 32) | uint32_t(e.w);
    }
  }
  // Squish: sort, keep the first key per neighbour id, drop self-loops.
  std::vector<int64_t> kept(V, 0);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t n = 0; n < V; ++n) {
    uint64_t *b = keys.data() + deg[n], *e = keys.data() + deg[n + 1];
    std::sort(b, e);
    int64_t k = 0;
    int64_t last = -1;
    for (uint64_t *p = b; p < e; ++p) {
      const int64_t id = int64_t(*p >> 32);
      if (id == last) continue;
      last = id;
      if (id == n) continue;
      b[k++] = *p;
    }
    kept[n] = k;
  }
  int64_t E = 0;
  for (int64_t n = 0; n < V; ++n) E += kept[n];
  if (E > std::numeric_limits<int32_t>::max())
    return gg::set_error(GG_ERR_INVALID,
                         "%lld edges exceed the int32 offsets of the CSR layout",
                         (long long)E);
  auto *g = new (std::nothrow) gg_host_graph();
  if (!g) return gg::set_error(GG_ERR_OOM, "host graph allocation failed");
  g->V = (int32_t)V;
  g->E = E;
  g->offsets.resize(V + 1);
  g->dst.resize(E);
  g->w.resize(E);
  int64_t run = 0;
  for (int64_t n = 0; n < V; ++n) {
    g->offsets[n] = (int32_t)run;
    run += kept[n];
  }
  g->offsets[V] = (int32_t)run;
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t n = 0; n < V; ++n) {
    const uint64_t *b = keys.data() + deg[n];
    int32_t o = g->offsets[n];
    for (int64_t k = 0; k < kept[n]; ++k) {
      g->dst[o + k] = int32_t(b[k] >> 32);
      g->w[o + k] = int32_t(uint32_t(b[k]));
    }
  }
  *out = g;
  return GG_OK;
}

// R-MAT edge list (generator.h:74-107 semantics).
void rmat_edges(int scale, int64_t num_edges, float A, float B, float C,
                int64_t seed, std::vector<WEdge> &el) {
  el.resize(num_edges);
  const float AB = A + B;     // float sums, as in the reference's comparisons
  const float ABC = A + B + C;
#pragma omp parallel
  {
    std::mt19937 rng;
    std::uniform_real_distribution<float> udist(0, 1.0f);
#pragma omp for schedule(static)
    for (int64_t block = 0; block < num_edges; block += kBlock) {
      rng.seed((std::mt19937::result_type)(seed + block / kBlock));
      const int64_t end = std::min(block + kBlock, num_edges);
      for (int64_t e = block; e < end; ++e) {
        int32_t src = 0, dst = 0;
        for (int depth = 0; depth < scale; ++depth) {
          const float r = udist(rng);
          src <<= 1;
          dst <<= 1;
          if (r < AB) {
            if (r > A) dst++;
          } else {
            src++;
            if (r > ABC) dst++;
          }
        }
        el[e].u = src;
        el[e].v = dst;
        el[e].w = 1;
      }
    }
  }
  // Id permutation: one std::mt19937(seed) driving std::shuffle over 0..N-1.
  const int64_t N = int64_t(1) << scale;
  std::vector<int32_t> perm(N);
  for (int64_t n = 0; n < N; ++n) perm[n] = (int32_t)n;
  std::mt19937 prng((std::mt19937::result_type)seed);
  std::shuffle(perm.begin(), perm.end(), prng);
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < num_edges; ++e) {
    el[e].u = perm[el[e].u];
    el[e].v = perm[el[e].v];
  }
}

// Block-reseeded uniform integer weights (generator.h:125-139 semantics).
template <class F>
void block_weights(int64_t n, int64_t seed, int32_t wmin, int32_t wmax, F &&set) {
#pragma omp parallel
  {
    std::mt19937 rng;
    std::uniform_int_distribution<int> udist(wmin, wmax);
#pragma omp for schedule(static)
    for (int64_t block = 0; block < n; block += kBlock) {
      rng.seed((std::mt19937::result_type)(seed + block / kBlock));
      const int64_t end = std::min(block + kBlock, n);
      for (int64_t e = block; e < end; ++e) set(e, (int32_t)udist(rng));
    }
  }
}

bool ends_with(const std::string &s, const char *suf) {
  const size_t n = strlen(suf);
  return s.size() >= n && s.compare(s.size() - n, n, suf) == 0;
}

gg_status load_bin(const std::string &path, gg_host_graph **out) {
  FILE *f = fopen(path.c_str(), "rb");
  if (!f) return gg::set_error(GG_ERR_IO, "cannot open %s: %s", path.c_str(), strerror(errno));
  int32_t hdr[2];
  if (fread(hdr, sizeof(int32_t), 2, f) != 2) {
    fclose(f);
    return gg::set_error(GG_ERR_IO, "%s: truncated header", path.c_str());
  }
  const int64_t V = hdr[0], E = hdr[1];
  fseek(f, 0, SEEK_END);
  const long long size = ftell(f);
  fseek(f, 8, SEEK_SET);
  const long long want = 8 + 12LL * E + 4LL * (V + 1);
  if (V <= 0 || E < 0 || size != want) {
    fclose(f);
    return gg::set_error(GG_ERR_IO,
                         "%s: size %lld does not match header V=%lld E=%lld "
                         "(expected %lld bytes)",
                         path.c_str(), size, (long long)V, (long long)E, want);
  }
  auto *g = new gg_host_graph();
  g->V = (int32_t)V;
  g->E = E;
  std::vector<int32_t> src(E);
  g->dst.resize(E);
  g->w.resize(E);
  g->offsets.resize(V + 1);
  bool ok = fread(src.data(), 4, E, f) == (size_t)E &&
            fread(&g->dst[0], 4, E, f) == (size_t)E &&
            fread(&g->w[0], 4, E, f) == (size_t)E &&
            fread(&g->offsets[0], 4, V + 1, f) == (size_t)(V + 1);
  fclose(f);
  if (!ok) {
    delete g;
    return gg::set_error(GG_ERR_IO, "%s: short read", path.c_str());
  }
  // Validate the CSR: monotone offsets covering [0,E], ids in range, and the
  // COO source column consistent with the offsets.
  bool valid = g->offsets[0] == 0 && g->offsets[V] == E;
  for (int64_t v = 0; valid && v < V; ++v) {
    if (g->offsets[v] > g->offsets[v + 1]) valid = false;
    for (int64_t k = g->offsets[v]; valid && k < g->offsets[v + 1]; ++k)
      if (src[k] != v || g->dst[k] < 0 || g->dst[k] >= V) valid = false;
  }
  if (!valid) {
    delete g;
    return gg::set_error(GG_ERR_IO, "%s: corrupt CSR contents", path.c_str());
  }
  *out = g;
  return GG_OK;
}

gg_status load_text(const std::string &path, bool symmetrize, gg_host_graph **out) {
  std::ifstream in(path);
  if (!in.is_open())
    return gg::set_error(GG_ERR_IO, "cannot open %s", path.c_str());
  std::vector<WEdge> el;
  int64_t max_id = -1;
  bool force_sym = false;
  auto push = [&](int64_t u, int64_t v, int64_t w) -> bool {
    if (u < 0 || v < 0 || u > INT32_MAX - 1 || v > INT32_MAX - 1) return false;
    el.push_back({(int32_t)u, (int32_t)v, (int32_t)w});
    max_id = std::max(max_id, std::max(u, v));
    return true;
  };
  std::string line;
  if (ends_with(path, ".el") || ends_with(path, ".wel")) {
    // reader.h:55-72: whitespace-separated "u v" or "u v w".
    const bool weighted = ends_with(path, ".wel");
    int64_t u, v, w = 1;
    while (in >> u >> v) {
      if (weighted && !(in >> w))
        return gg::set_error(GG_ERR_IO, "%s: truncated weighted edge", path.c_str());
      if (!push(u, v, w)) return gg::set_error(GG_ERR_IO, "%s: bad vertex id", path.c_str());
    }
  } else if (ends_with(path, ".gr")) {
    // reader.h:74-87: DIMACS "a u v w" lines; ids are kept as written.
    while (std::getline(in, line)) {
      if (line.empty() || line[0] != 'a') continue;
      std::istringstream ls(line.substr(1));
      int64_t u, v, w;
      if (!(ls >> u >> v >> w)) return gg::set_error(GG_ERR_IO, "%s: bad arc line", path.c_str());
      if (!push(u, v, w)) return gg::set_error(GG_ERR_IO, "%s: bad vertex id", path.c_str());
    }
  } else if (ends_with(path, ".mtx")) {
    // reader.h:137-200: MatrixMarket coordinate, 1-based ids, symmetric => both.
    std::string start, object, format, field, symmetry;
    in >> start >> object >> format >> field >> symmetry;
    if (start != "%%MatrixMarket" || object != "matrix" || format != "coordinate")
      return gg::set_error(GG_ERR_IO, "%s: not a MatrixMarket coordinate file", path.c_str());
    const bool weighted = field != "pattern";
    force_sym = symmetry == "symmetric";
    std::getline(in, line);
    while (in.peek() == '%') std::getline(in, line);
    int64_t m, n, nnz;
    if (!(in >> m >> n >> nnz) || m != n)
      return gg::set_error(GG_ERR_IO, "%s: bad or non-square size line", path.c_str());
    for (int64_t i = 0; i < nnz; ++i) {
      int64_t u, v;
      double w = 1;
      if (!(in >> u >> v)) return gg::set_error(GG_ERR_IO, "%s: truncated entries", path.c_str());
      if (weighted && !(in >> w)) return gg::set_error(GG_ERR_IO, "%s: truncated weight", path.c_str());
      if (!push(u - 1, v - 1, (int64_t)w)) return gg::set_error(GG_ERR_IO, "%s: bad id", path.c_str());
    }
    max_id = std::max(max_id, m - 1);
  } else {
    return gg::set_error(GG_ERR_IO, "%s: unknown graph file suffix", path.c_str());
  }
  if (max_id < 0) return gg::set_error(GG_ERR_IO, "%s: no edges", path.c_str());
  return build_csr(max_id + 1, el, symmetrize || force_sym, out);
}

// GAPBS serialized graphs (infra_gapbs/reader.h:322-369, writer.h:39-70):
//   [bool directed][i64 num_edges][i64 num_nodes][i64 offsets[V+1]][neighbours[E]]
//   and, when directed, the in-lists in the same two arrays again.
// A .sg neighbour is an int32 id, a .wsg one an {int32 id, int32 weight} pair.
// The out-lists are taken as they are stored (GAPBS writes squished graphs);
// the in-lists are skipped.
gg_status load_sg(const std::string &path, bool weighted, gg_host_graph **out) {
  FILE *f = fopen(path.c_str(), "rb");
  if (!f) return gg::set_error(GG_ERR_IO, "cannot open %s: %s", path.c_str(), strerror(errno));
  unsigned char directed = 0;
  int64_t E = 0, V = 0;
  const bool hdr = fread(&directed, 1, 1, f) == 1 && fread(&E, 8, 1, f) == 1 && fread(&V, 8, 1, f) == 1;
  fseek(f, 0, SEEK_END);
  const long long size = ftell(f);
  const long long nb = weighted ? 8 : 4;
  const long long one = 8LL * (V + 1) + nb * E;
  if (!hdr || directed > 1 || V <= 0 || V > INT32_MAX - 1 || E < 0 || E > INT32_MAX ||
      size != 17 + one * (directed ? 2 : 1)) {
    fclose(f);
    return gg::set_error(GG_ERR_IO, "%s: header (V=%lld, E=%lld) does not match the file size %lld",
                         path.c_str(), (long long)V, (long long)E, size);
  }
  fseek(f, 17, SEEK_SET);
  std::vector<int64_t> off(V + 1);
  std::vector<int32_t> nbr((size_t)E * (weighted ? 2 : 1));
  const bool ok = fread(off.data(), 8, V + 1, f) == (size_t)(V + 1) &&
                  fread(nbr.data(), nb, E, f) == (size_t)E;
  fclose(f);
  if (!ok) return gg::set_error(GG_ERR_IO, "%s: short read", path.c_str());
  bool valid = off[0] == 0 && off[V] == E;
  for (int64_t v = 0; valid && v < V; ++v) valid = off[v] <= off[v + 1];
  auto *g = new (std::nothrow) gg_host_graph();
  if (!g) return gg::set_error(GG_ERR_OOM, "host graph allocation failed");
  g->V = (int32_t)V;
  g->E = E;
  g->offsets.resize(V + 1);
  g->dst.resize(E);
  g->w.resize(E);
  for (int64_t v = 0; valid && v <= V; ++v) g->offsets[v] = (int32_t)off[v];
  for (int64_t k = 0; valid && k < E; ++k) {
    const int32_t d = weighted ? nbr[2 * k] : nbr[k];
    valid = d >= 0 && d < V;
    g->dst[k] = d;
    g->w[k] = weighted ? nbr[2 * k + 1] : 1;
  }
  if (!valid) {
    delete g;
    return gg::set_error(GG_ERR_IO, "%s: corrupt offsets or neighbour ids", path.c_str());
  }
  *out = g;
  return GG_OK;
}

}  // namespace

extern "C" {

gg_status gg_host_graph_save_sg(const gg_host_graph *g, const char *path, int32_t directed) {
  GG_CHECK_ARG(g && path, "bad arguments");
  const std::string p(path);
  const bool weighted = ends_with(p, ".wsg");
  GG_CHECK_ARG(weighted || ends_with(p, ".sg"), "a serialized graph file ends in .sg or .wsg");
  const int64_t V = g->V, E = g->E;
  std::vector<int64_t> off(V + 1);
  auto lists = [&](const int32_t *o, const int32_t *d, const int32_t *w, std::vector<int32_t> &buf) {
    for (int64_t v = 0; v <= V; ++v) off[v] = o[v];
    buf.resize((size_t)E * (weighted ? 2 : 1));
    for (int64_t k = 0; k < E; ++k) {
      if (weighted) {
        buf[2 * k] = d[k];
        buf[2 * k + 1] = w[k];
      } else {
        buf[k] = d[k];
      }
    }
  };
  FILE *f = fopen(path, "wb");
  if (!f) return gg::set_error(GG_ERR_IO, "cannot create %s: %s", path, strerror(errno));
  const unsigned char dir = directed ? 1 : 0;
  std::vector<int32_t> buf;
  lists(g->offsets.data(), g->dst.data(), g->w.data(), buf);
  const size_t nb = weighted ? 8 : 4;
  bool ok = fwrite(&dir, 1, 1, f) == 1 && fwrite(&E, 8, 1, f) == 1 && fwrite(&V, 8, 1, f) == 1 &&
            fwrite(off.data(), 8, V + 1, f) == (size_t)(V + 1) && fwrite(buf.data(), nb, E, f) == (size_t)E;
  if (ok && directed) {
    // in-lists: sources of each vertex's in-edges in ascending order, with weights
    std::vector<int32_t> io(V + 1, 0), isrc(E), iw(E);
    for (int64_t k = 0; k < E; ++k) io[g->dst[k] + 1]++;
    for (int64_t v = 0; v < V; ++v) io[v + 1] += io[v];
    std::vector<int32_t> pos(io.begin(), io.end() - 1);
    for (int64_t u = 0; u < V; ++u)
      for (int64_t k = g->offsets[u]; k < g->offsets[u + 1]; ++k) {
        isrc[pos[g->dst[k]]] = (int32_t)u;
        iw[pos[g->dst[k]]++] = g->w[k];
      }
    lists(io.data(), isrc.data(), iw.data(), buf);
    ok = fwrite(off.data(), 8, V + 1, f) == (size_t)(V + 1) && fwrite(buf.data(), nb, E, f) == (size_t)E;
  }
  ok = (fclose(f) == 0) && ok;
  if (!ok) return gg::set_error(GG_ERR_IO, "short write to %s", path);
  return GG_OK;
}

gg_status gg_host_graph_rmat(int32_t scale, int32_t degree, float a, float b,
                             float c, int64_t seed, int32_t symmetrize,
                             int32_t wmin, int32_t wmax, gg_host_graph **out) {
  GG_CHECK_ARG(out, "out is NULL");
  GG_CHECK_ARG(scale >= 1 && scale <= 30, "scale must be in [1,30]");
  GG_CHECK_ARG(degree >= 1, "degree must be >= 1");
  GG_CHECK_ARG(a >= 0 && b >= 0 && c >= 0 && a + b + c <= 1.0f, "bad R-MAT probabilities");
  GG_CHECK_ARG(wmin >= 1 && wmax >= wmin, "bad weight range");
  const int64_t num_edges = (int64_t(1) << scale) * degree;
  std::vector<WEdge> el;
  rmat_edges(scale, num_edges, a, b, c, seed, el);
  block_weights(num_edges, seed, wmin, wmax,
                [&](int64_t e, int32_t w) { el[e].w = w; });
  // The vertex count is the largest id seen + 1, as BuilderBase::MakeGraphFromEL
  // sizes a generated graph (builder.h:62-71, 210-211).
  int32_t max_id = 0;
#pragma omp parallel for reduction(max : max_id) schedule(static)
  for (int64_t e = 0; e < num_edges; ++e) max_id = std::max(max_id, std::max(el[e].u, el[e].v));
  return build_csr((int64_t)max_id + 1, el, symmetrize != 0, out);
}

gg_status gg_host_graph_grid(int32_t rows, int32_t cols, int64_t seed,
                             int32_t wmin, int32_t wmax, gg_host_graph **out) {
  GG_CHECK_ARG(out, "out is NULL");
  GG_CHECK_ARG(rows >= 1 && cols >= 1, "rows and cols must be >= 1");
  GG_CHECK_ARG((int64_t)rows * cols < INT32_MAX, "grid too large for int32 ids");
  GG_CHECK_ARG(wmin >= 1 && wmax >= wmin, "bad weight range");
  const int64_t V = (int64_t)rows * cols;
  auto *g = new (std::nothrow) gg_host_graph();
  if (!g) return gg::set_error(GG_ERR_OOM, "host graph allocation failed");
  g->V = (int32_t)V;
  g->offsets.resize(V + 1);
  // Degree of (r,c): neighbours up, left, right, down that exist.
  std::vector<int64_t> off(V + 1);
  for (int64_t v = 0; v < V; ++v) {
    const int64_t r = v / cols, q = v % cols;
    off[v] = (r > 0) + (q > 0) + (q + 1 < cols) + (r + 1 < rows);
  }
  int64_t run = 0;
  for (int64_t v = 0; v < V; ++v) {
    const int64_t d = off[v];
    g->offsets[v] = (int32_t)run;
    run += d;
  }
  g->offsets[V] = (int32_t)run;
  g->E = run;
  g->dst.resize(run);
  g->w.resize(run);
#pragma omp parallel for schedule(static)
  for (int64_t v = 0; v < V; ++v) {
    const int64_t r = v / cols, q = v % cols;
    int32_t k = g->offsets[v];
    if (r > 0) g->dst[k++] = (int32_t)(v - cols);  // ascending neighbour ids
    if (q > 0) g->dst[k++] = (int32_t)(v - 1);
    if (q + 1 < cols) g->dst[k++] = (int32_t)(v + 1);
    if (r + 1 < rows) g->dst[k++] = (int32_t)(v + cols);
  }
  block_weights(run, seed, wmin, wmax, [&](int64_t e, int32_t w) { g->w[e] = w; });
  *out = g;
  return GG_OK;
}

gg_status gg_host_graph_from_edges(int32_t num_vertices, int64_t num_edges,
                                   const int32_t *u, const int32_t *v,
                                   const int32_t *w, int32_t symmetrize,
                                   gg_host_graph **out) {
  GG_CHECK_ARG(out && num_vertices > 0 && num_edges >= 0, "bad arguments");
  GG_CHECK_ARG(num_edges == 0 || (u && v), "edge arrays are NULL");
  std::vector<WEdge> el(num_edges);
  for (int64_t i = 0; i < num_edges; ++i) el[i] = {u[i], v[i], w ? w[i] : 1};
  return build_csr(num_vertices, el, symmetrize != 0, out);
}

gg_status gg_host_graph_from_csr(int32_t num_vertices, int64_t num_edges,
                                 const int32_t *offsets, const int32_t *dst,
                                 const int32_t *weights, gg_host_graph **out) {
  GG_CHECK_ARG(out && num_vertices > 0 && num_edges >= 0 && offsets, "bad arguments");
  GG_CHECK_ARG(num_edges == 0 || dst, "dst is NULL");
  GG_CHECK_ARG(num_edges <= INT32_MAX, "too many edges for int32 offsets");
  if (offsets[0] != 0 || offsets[num_vertices] != num_edges)
    return gg::set_error(GG_ERR_INVALID, "offsets must start at 0 and end at E");
  for (int32_t i = 0; i < num_vertices; ++i)
    if (offsets[i] > offsets[i + 1])
      return gg::set_error(GG_ERR_INVALID, "offsets not monotone at %d", i);
  for (int64_t e = 0; e < num_edges; ++e)
    if (dst[e] < 0 || dst[e] >= num_vertices)
      return gg::set_error(GG_ERR_INVALID, "dst[%lld] out of range", (long long)e);
  auto *g = new gg_host_graph();
  g->V = num_vertices;
  g->E = num_edges;
  g->offsets.assign(offsets, offsets + num_vertices + 1);
  g->dst.assign(dst, dst + num_edges);
  if (weights)
    g->w.assign(weights, weights + num_edges);
  else
    g->w.assign(num_edges, 1);
  *out = g;
  return GG_OK;
}

gg_status gg_host_graph_load(const char *path, int32_t symmetrize, gg_host_graph **out) {
  GG_CHECK_ARG(path && out, "bad arguments");
  const std::string p(path);
  if (ends_with(p, ".graphit_bin")) return load_bin(p, out);
  if (ends_with(p, ".sg") || ends_with(p, ".wsg")) return load_sg(p, ends_with(p, ".wsg"), out);
  return load_text(p, symmetrize != 0, out);
}

gg_status gg_host_graph_save_bin(const gg_host_graph *g, const char *path) {
  GG_CHECK_ARG(g && path, "bad arguments");
  GG_CHECK_ARG(g->E <= INT32_MAX, "too many edges for the int32 header");
  FILE *f = fopen(path, "wb");
  if (!f) return gg::set_error(GG_ERR_IO, "cannot create %s: %s", path, strerror(errno));
  const int32_t hdr[2] = {g->V, (int32_t)g->E};
  std::vector<int32_t> src(g->E);
  for (int32_t v = 0; v < g->V; ++v)
    for (int32_t k = g->offsets[v]; k < g->offsets[v + 1]; ++k) src[k] = v;
  bool ok = fwrite(hdr, 4, 2, f) == 2 &&
            fwrite(src.data(), 4, g->E, f) == (size_t)g->E &&
            fwrite(g->dst.data(), 4, g->E, f) == (size_t)g->E &&
            fwrite(g->w.data(), 4, g->E, f) == (size_t)g->E &&
            fwrite(g->offsets.data(), 4, g->V + 1, f) == (size_t)(g->V + 1);
  ok = (fclose(f) == 0) && ok;
  if (!ok) return gg::set_error(GG_ERR_IO, "short write to %s", path);
  return GG_OK;
}

gg_status gg_host_graph_union(const gg_host_graph *const *parts, int32_t n, int32_t *vertex_offsets,
                              gg_host_graph **out) {
  GG_CHECK_ARG(parts && n >= 1 && out, "bad arguments");
  int64_t V = 0, E = 0;
  for (int32_t i = 0; i < n; ++i) {
    GG_CHECK_ARG(parts[i], "NULL part");
    V += parts[i]->V;
    E += parts[i]->E;
  }
  if (V >= INT32_MAX || E > INT32_MAX)
    return gg::set_error(GG_ERR_INVALID, "union of %d graphs exceeds the int32 CSR layout", n);
  auto *g = new (std::nothrow) gg_host_graph();
  if (!g) return gg::set_error(GG_ERR_OOM, "host graph allocation failed");
  g->V = (int32_t)V;
  g->E = E;
  g->offsets.resize(V + 1);
  g->dst.resize(E);
  g->w.resize(E);
  int32_t vb = 0, eb = 0;
  for (int32_t i = 0; i < n; ++i) {
    const gg_host_graph *p = parts[i];
    if (vertex_offsets) vertex_offsets[i] = vb;
    for (int32_t v = 0; v < p->V; ++v) g->offsets[vb + v] = eb + p->offsets[v];
    for (int64_t e = 0; e < p->E; ++e) {
      g->dst[eb + e] = vb + p->dst[e];
      g->w[eb + e] = p->w[e];
    }
    vb += p->V;
    eb += (int32_t)p->E;
  }
  g->offsets[V] = eb;
  if (vertex_offsets) vertex_offsets[n] = vb;
  *out = g;
  return GG_OK;
}

gg_status gg_host_graph_pick_sources(const gg_host_graph *g, int32_t n, int64_t seed, int32_t *out) {
  GG_CHECK_ARG(g && out && n >= 0, "bad arguments");
  if (g->E == 0) return gg::set_error(GG_ERR_INVALID, "graph has no edges to pick sources from");
  // SourcePicker::PickNext (infra_gapbs/benchmark.h:50-71): uniform ids from one
  // std::mt19937, rejecting vertices without out-edges.
  std::mt19937 rng((std::mt19937::result_type)seed);
  std::uniform_int_distribution<int32_t> udist(0, g->V - 1);
  for (int32_t i = 0; i < n; ++i) {
    int32_t s;
    do {
      s = udist(rng);
    } while (g->offsets[s + 1] == g->offsets[s]);
    out[i] = s;
  }
  return GG_OK;
}

gg_status gg_host_graph_mix_spec(int64_t seed, int32_t count, int32_t *spec) {
  GG_CHECK_ARG(spec && count >= 0, "bad arguments");
  // One std::mt19937(seed) draws, per graph, a kind (grid with probability
  // 1/4), then a grid side 2^[8,11] or an R-MAT scale [12,20] and edge factor
  // [4,32]; each graph's own generator seed is seed + 1 + its index.
  std::mt19937 rng((std::mt19937::result_type)seed);
  std::uniform_int_distribution<int32_t> kind(0, 3), side(8, 11), scale(12, 20), ef(4, 32);
  for (int32_t i = 0; i < count; ++i) {
    int32_t *r = spec + 3 * (size_t)i;
    if (kind(rng) == 0) {
      r[0] = 1;
      r[1] = 1 << side(rng);
      r[2] = 0;
    } else {
      r[0] = 0;
      r[1] = scale(rng);
      r[2] = ef(rng);
    }
  }
  return GG_OK;
}

gg_status gg_host_graph_info(const gg_host_graph *g, int32_t *num_vertices, int64_t *num_edges) {
  GG_CHECK_ARG(g, "graph is NULL");
  if (num_vertices) *num_vertices = g->V;
  if (num_edges) *num_edges = g->E;
  return GG_OK;
}

const int32_t *gg_host_graph_offsets(const gg_host_graph *g) { return g ? g->offsets.data() : nullptr; }
const int32_t *gg_host_graph_dst(const gg_host_graph *g) { return g ? g->dst.data() : nullptr; }
const int32_t *gg_host_graph_weights(const gg_host_graph *g) { return g ? g->w.data() : nullptr; }
void gg_host_graph_destroy(gg_host_graph *g) { delete g; }

}  // extern "C"
