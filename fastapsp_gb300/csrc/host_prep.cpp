// host_prep.cpp -- host-side preprocessing of the Fast-APSP engine: the
// MatrixMarket reader, the K-way partitioner and the boundary/reorder step.
// Pure C++ (no CUDA); exported through the C ABI in include/fastapsp.h.

#include <sys/stat.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <numeric>
#include <random>
#include <string>
#include <thread>
#include <vector>

#include "fap_internal.h"

namespace fapi {

// ---------------------------------------------------------------------------
// MatrixMarket reader.  Same semantics as the reference's readVerEdges /
// readMatFile (fap/utils/readMatFile.h:36-173): leading '%' lines skipped,
// header "n n m", 1-based ids, undirected lines doubled, |w|, unweighted -> 1,
// rows in reverse input order.  The body is parsed from one buffer read.
// ---------------------------------------------------------------------------
namespace {

struct Buf {
  std::vector<char> data;
  size_t pos = 0;
};

bool slurp(const char *path, Buf &b) {
  FILE *f = std::fopen(path, "rb");
  if (!f) return false;
  std::fseek(f, 0, SEEK_END);
  long sz = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  b.data.resize((size_t)std::max(0L, sz) + 1);
  size_t got = std::fread(b.data.data(), 1, (size_t)std::max(0L, sz), f);
  std::fclose(f);
  b.data[got] = '\0';
  b.data.resize(got + 1);
  return true;
}

void skip_comment_lines(Buf &b) {
  while (b.pos < b.data.size() - 1 && b.data[b.pos] == '%') {
    while (b.pos < b.data.size() - 1 && b.data[b.pos] != '\n') b.pos++;
    if (b.pos < b.data.size() - 1) b.pos++;
  }
}

bool next_ll(Buf &b, long long &v) {
  char *p = b.data.data() + b.pos;
  char *end = nullptr;
  while (*p && std::isspace((unsigned char)*p)) p++;
  if (!*p) return false;
  v = std::strtoll(p, &end, 10);
  if (end == p) return false;
  b.pos = (size_t)(end - b.data.data());
  return true;
}

bool next_double(Buf &b, double &v) {
  char *p = b.data.data() + b.pos;
  char *end = nullptr;
  while (*p && std::isspace((unsigned char)*p)) p++;
  if (!*p) return false;
  v = std::strtod(p, &end);
  if (end == p) return false;
  b.pos = (size_t)(end - b.data.data());
  return true;
}

// Binary CSR cache beside the .mtx file (<path>.fapcsr): the reader's
// output for one (directed, weighted) reading of one version of the file,
// so that later reads skip the text parse.  Layout (host byte order):
//   char magic[8] = "FAPCSR01"; int32 directed, weighted; uint64 source size;
//   int64 source mtime (s), mtime (ns); int32 n; int64 header m; int64 m;
//   int32 row_offset[n + 1]; int32 col_val[m]; float weight[m].
// A cache is used only when every header field matches the file as it is now;
// otherwise the file is parsed and the cache rewritten (through a temporary
// file and a rename).  FAP_MTX_CACHE=0 in the environment turns it off.
struct CacheHead {
  char magic[8];
  int32_t directed, weighted;
  uint64_t src_size;
  int64_t src_sec, src_nsec;
  int32_t n;
  int64_t header_m, m;
};

bool cache_enabled() {
  const char *v = std::getenv("FAP_MTX_CACHE");
  return !(v && v[0] == '0');
}

std::string cache_path(const char *path) { return std::string(path) + ".fapcsr"; }

bool source_stamp(const char *path, uint64_t &size, int64_t &sec, int64_t &nsec) {
  struct stat st;
  if (stat(path, &st) != 0) return false;
  size = (uint64_t)st.st_size;
  sec = (int64_t)st.st_mtim.tv_sec;
  nsec = (int64_t)st.st_mtim.tv_nsec;
  return true;
}

// Opens the cache of `path` and reads its header when it matches the file
// as it is now; returns the open stream (positioned after the header) or null.
FILE *open_cache(const char *path, bool directed, bool weighted, CacheHead &h) {
  if (!cache_enabled()) return nullptr;
  uint64_t size;
  int64_t sec, nsec;
  if (!source_stamp(path, size, sec, nsec)) return nullptr;
  FILE *f = std::fopen(cache_path(path).c_str(), "rb");
  if (!f) return nullptr;
  if (std::fread(&h, sizeof(h), 1, f) != 1 || std::memcmp(h.magic, "FAPCSR01", 8) != 0 ||
      h.directed != (int32_t)directed || h.weighted != (int32_t)weighted || h.src_size != size ||
      h.src_sec != sec || h.src_nsec != nsec || h.n < 0 || h.m < 0 || h.m > h.header_m) {
    std::fclose(f);
    return nullptr;
  }
  return f;
}

void write_cache(const char *path, bool directed, bool weighted, int32_t n, int64_t header_m,
                 int64_t m, const int32_t *row_offset, const int32_t *col_val, const float *weight) {
  if (!cache_enabled()) return;
  CacheHead h{};
  std::memcpy(h.magic, "FAPCSR01", 8);
  h.directed = directed;
  h.weighted = weighted;
  if (!source_stamp(path, h.src_size, h.src_sec, h.src_nsec)) return;
  h.n = n;
  h.header_m = header_m;
  h.m = m;
  const std::string fin = cache_path(path), tmp = fin + ".tmp";
  FILE *f = std::fopen(tmp.c_str(), "wb");
  if (!f) return;  // read-only directory: no cache
  bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1 &&
            std::fwrite(row_offset, sizeof(int32_t), (size_t)n + 1, f) == (size_t)n + 1 &&
            std::fwrite(col_val, sizeof(int32_t), (size_t)m, f) == (size_t)m &&
            std::fwrite(weight, sizeof(float), (size_t)m, f) == (size_t)m;
  ok = std::fclose(f) == 0 && ok;
  if (!ok || std::rename(tmp.c_str(), fin.c_str()) != 0) std::remove(tmp.c_str());
}

// The body's entries parsed by up to 16 threads, each over a run of whole
// lines; concatenated in input order.
struct Entries {
  std::vector<int32_t> src, dst;
  std::vector<float> w;
  int bad = 0;  // 1: vertex id outside 1..n
};

void parse_lines(const char *p, const char *end, bool directed, bool weighted, int32_t n, Entries &out) {
  while (p < end) {
    char *q = nullptr;
    while (p < end && std::isspace((unsigned char)*p)) p++;
    if (p >= end) break;
    const long long a = std::strtoll(p, &q, 10);
    if (q == p) break;
    p = q;
    const long long c2 = std::strtoll(p, &q, 10);
    if (q == p) break;
    p = q;
    double c = 1.0;
    if (weighted) {
      c = std::strtod(p, &q);
      if (q == p) break;
      p = q;
    }
    if (a < 1 || a > n || c2 < 1 || c2 > n) {
      out.bad = 1;
      return;
    }
    const float tc = weighted ? (float)std::fabs(c) : 1.0f;
    out.src.push_back((int32_t)(a - 1));
    out.dst.push_back((int32_t)(c2 - 1));
    out.w.push_back(tc);
    if (!directed) {
      out.src.push_back((int32_t)(c2 - 1));
      out.dst.push_back((int32_t)(a - 1));
      out.w.push_back(tc);
    }
  }
}

}  // namespace

int mtx_counts(const char *path, bool directed, int32_t *n, int64_t *m) {
  CacheHead h;
  // the cache records the flags it was read with; either reading gives the header counts
  FILE *cf = open_cache(path, directed, false, h);
  if (!cf) cf = open_cache(path, directed, true, h);
  if (cf) {
    std::fclose(cf);
    *n = h.n;
    *m = h.header_m;
    return FAP_OK;
  }
  Buf b;
  if (!slurp(path, b)) return set_error(FAP_ERR_IO, std::string("cannot open ") + path);
  skip_comment_lines(b);
  long long nn, t, mm;
  if (!next_ll(b, nn) || !next_ll(b, t) || !next_ll(b, mm))
    return set_error(FAP_ERR_IO, "bad MatrixMarket header");
  if (nn < 0 || nn > INT32_MAX || mm < 0) return set_error(FAP_ERR_RANGE, "header out of range");
  *n = (int32_t)nn;
  *m = directed ? (int64_t)mm : 2 * (int64_t)mm;
  return FAP_OK;
}

int mtx_read(const char *path, bool directed, bool weighted, int32_t n, int64_t m,
             int32_t *adj_size, int32_t *row_offset, int32_t *col_val, float *weight) {
  {
    CacheHead h;
    if (FILE *cf = open_cache(path, directed, weighted, h)) {
      bool ok = h.n == n && h.m <= m &&
                std::fread(row_offset, sizeof(int32_t), (size_t)n + 1, cf) == (size_t)n + 1 &&
                std::fread(col_val, sizeof(int32_t), (size_t)h.m, cf) == (size_t)h.m &&
                std::fread(weight, sizeof(float), (size_t)h.m, cf) == (size_t)h.m;
      std::fclose(cf);
      if (ok) {
        for (int32_t i = 0; i < n; i++) adj_size[i] = row_offset[i + 1] - row_offset[i];
        return FAP_OK;
      }  // a damaged cache: parse the file (and rewrite the cache) below
    }
  }
  Buf b;
  if (!slurp(path, b)) return set_error(FAP_ERR_IO, std::string("cannot open ") + path);
  skip_comment_lines(b);
  long long nn, t, mm;
  if (!next_ll(b, nn) || !next_ll(b, t) || !next_ll(b, mm))
    return set_error(FAP_ERR_IO, "bad MatrixMarket header");
  // Entries in input order (threads over runs of whole lines, concatenated
  // in order); each row is emitted newest-first afterwards.
  const char *body = b.data.data() + b.pos, *body_end = b.data.data() + b.data.size() - 1;
  const size_t len = (size_t)(body_end - body);
  const int nt = (int)std::max<size_t>(1, std::min<size_t>({16, std::thread::hardware_concurrency() ? std::thread::hardware_concurrency() : 1, len / (1 << 20)}));
  std::vector<const char *> cuts(nt + 1, body_end);
  cuts[0] = body;
  for (int i = 1; i < nt; i++) {
    const char *c = body + len * i / nt;
    while (c < body_end && *c != '\n') c++;
    cuts[i] = std::max(c, cuts[i - 1]);
  }
  std::vector<Entries> parts(nt);
  {
    std::vector<std::thread> th;
    for (int i = 1; i < nt; i++)
      th.emplace_back(parse_lines, cuts[i], cuts[i + 1], directed, weighted, n, std::ref(parts[i]));
    parse_lines(cuts[0], cuts[1], directed, weighted, n, parts[0]);
    for (auto &x : th) x.join();
  }
  size_t total = 0;
  for (const Entries &p : parts) {
    if (p.bad) return set_error(FAP_ERR_RANGE, "vertex id outside 1..n in MatrixMarket body");
    total += p.src.size();
  }
  std::vector<int32_t> src, dst;
  std::vector<float> w;
  src.reserve(total);
  dst.reserve(total);
  w.reserve(total);
  for (Entries &p : parts) {
    src.insert(src.end(), p.src.begin(), p.src.end());
    dst.insert(dst.end(), p.dst.begin(), p.dst.end());
    w.insert(w.end(), p.w.begin(), p.w.end());
    p = Entries();  // release the part's buffers
  }
  if ((int64_t)src.size() > m) return set_error(FAP_ERR_RANGE, "more entries than the header announces");
  std::vector<int64_t> cnt((size_t)n + 1, 0);
  for (int32_t s : src) cnt[s + 1]++;
  row_offset[0] = 0;
  for (int32_t i = 0; i < n; i++) {
    adj_size[i] = (int32_t)cnt[i + 1];
    row_offset[i + 1] = row_offset[i] + (int32_t)cnt[i + 1];
  }
  // fill each row from its end backwards in input order -> newest first
  std::vector<int64_t> fill((size_t)n);
  for (int32_t i = 0; i < n; i++) fill[i] = row_offset[i + 1];
  for (size_t e = 0; e < src.size(); e++) {
    int64_t pos = --fill[src[e]];
    col_val[pos] = dst[e];
    weight[pos] = w[e];
  }
  write_cache(path, directed, weighted, n, directed ? (int64_t)mm : 2 * (int64_t)mm, (int64_t)src.size(),
              row_offset, col_val, weight);
  return FAP_OK;
}

// ---------------------------------------------------------------------------
// Multilevel K-way partitioner.  The reference calls METIS_PartGraphKway on
// the symmetrized graph (fap/utils/readIdFile.h:200-283); METIS is not part of
// this engine, so the same job (balanced parts, small edge cut) is done here:
//   1. coarsen by heavy-edge matching until ~40 vertices per part remain,
//   2. partition the coarsest graph by recursive greedy-growing bisection
//      with 2-way boundary refinement,
//   3. project back level by level with greedy K-way boundary refinement.
// Imbalance tolerance 3% (the reference's KaHIP setting, readIdFile.h:244).
// ---------------------------------------------------------------------------
namespace {

struct WGraph {
  int32_t n = 0;
  std::vector<int64_t> xadj;
  std::vector<int32_t> adj;
  std::vector<int32_t> ew;  // edge weights
  std::vector<int32_t> vw;  // vertex weights
};

WGraph symmetrize(int32_t n, const int32_t *ro, const int32_t *col) {
  std::vector<std::vector<int32_t>> nb(n);
  for (int32_t u = 0; u < n; u++)
    for (int32_t j = ro[u]; j < ro[u + 1]; j++) {
      int32_t v = col[j];
      if (v == u || v < 0 || v >= n) continue;
      nb[u].push_back(v);
      nb[v].push_back(u);
    }
  WGraph g;
  g.n = n;
  g.xadj.assign((size_t)n + 1, 0);
  g.vw.assign(n, 1);
  for (int32_t u = 0; u < n; u++) {
    auto &l = nb[u];
    std::sort(l.begin(), l.end());
    int32_t last = -1;
    for (int32_t v : l) {
      if (v == last) {
        g.ew.back() += 1;
        continue;
      }
      g.adj.push_back(v);
      g.ew.push_back(1);
      last = v;
    }
    g.xadj[u + 1] = (int64_t)g.adj.size();
  }
  return g;
}

// Heavy-edge matching; returns the coarse graph and the fine->coarse map.
WGraph coarsen(const WGraph &g, std::vector<int32_t> &cmap, std::mt19937_64 &rng,
               int64_t max_vw) {
  const int32_t n = g.n;
  std::vector<int32_t> match(n, -1), order(n);
  std::iota(order.begin(), order.end(), 0);
  std::shuffle(order.begin(), order.end(), rng);
  for (int32_t u : order) {
    if (match[u] != -1) continue;
    int32_t best = -1, bw = -1;
    for (int64_t j = g.xadj[u]; j < g.xadj[u + 1]; j++) {
      int32_t v = g.adj[j];
      if (match[v] != -1 || v == u) continue;
      if ((int64_t)g.vw[u] + g.vw[v] > max_vw) continue;
      if (g.ew[j] > bw) {
        bw = g.ew[j];
        best = v;
      }
    }
    if (best >= 0) {
      match[u] = best;
      match[best] = u;
    } else {
      match[u] = u;
    }
  }
  cmap.assign(n, -1);
  int32_t nc = 0;
  for (int32_t u = 0; u < n; u++) {
    if (cmap[u] != -1) continue;
    cmap[u] = nc;
    if (match[u] != u) cmap[match[u]] = nc;
    nc++;
  }
  WGraph c;
  c.n = nc;
  c.vw.assign(nc, 0);
  c.xadj.assign((size_t)nc + 1, 0);
  std::vector<int32_t> members_start(nc + 1, 0), members(n);
  for (int32_t u = 0; u < n; u++) members_start[cmap[u] + 1]++;
  for (int32_t i = 0; i < nc; i++) members_start[i + 1] += members_start[i];
  {
    std::vector<int32_t> fillp(members_start.begin(), members_start.end() - 1);
    for (int32_t u = 0; u < n; u++) members[fillp[cmap[u]]++] = u;
  }
  std::vector<int32_t> mark(nc, -1), slot(nc, 0);
  for (int32_t cu = 0; cu < nc; cu++) {
    int64_t base = (int64_t)c.adj.size();
    for (int32_t mi = members_start[cu]; mi < members_start[cu + 1]; mi++) {
      int32_t u = members[mi];
      c.vw[cu] += g.vw[u];
      for (int64_t j = g.xadj[u]; j < g.xadj[u + 1]; j++) {
        int32_t cv = cmap[g.adj[j]];
        if (cv == cu) continue;
        if (mark[cv] != cu) {
          mark[cv] = cu;
          slot[cv] = (int32_t)(c.adj.size() - base);
          c.adj.push_back(cv);
          c.ew.push_back(g.ew[j]);
        } else {
          c.ew[base + slot[cv]] += g.ew[j];
        }
      }
    }
    c.xadj[cu + 1] = (int64_t)c.adj.size();
  }
  return c;
}

// Greedy growing bisection of the vertex subset `verts` of g into side 0 with
// weight ~target0 and side 1 with the rest; followed by a 2-way refinement.
void bisect(const WGraph &g, const std::vector<int32_t> &verts, int64_t target0,
            std::vector<int32_t> &side, std::mt19937_64 &rng, int tries) {
  const int32_t nv = (int32_t)verts.size();
  std::vector<int32_t> local(g.n, -1);
  for (int32_t i = 0; i < nv; i++) local[verts[i]] = i;
  int64_t total = 0;
  for (int32_t v : verts) total += g.vw[v];
  std::vector<int32_t> best_side(nv, 1);
  int64_t best_cut = INT64_MAX;
  std::vector<int32_t> cur(nv), queue(nv), dist(nv);
  for (int t = 0; t < tries; t++) {
    // seed: a pseudo-peripheral vertex (two BFS sweeps from a random start)
    int32_t start = (int32_t)(rng() % (uint64_t)nv);
    for (int sweep = 0; sweep < 2; sweep++) {
      std::fill(dist.begin(), dist.end(), -1);
      int32_t qh = 0, qt = 0, last = start;
      dist[start] = 0;
      queue[qt++] = start;
      while (qh < qt) {
        int32_t li = queue[qh++];
        last = li;
        int32_t u = verts[li];
        for (int64_t j = g.xadj[u]; j < g.xadj[u + 1]; j++) {
          int32_t lv = local[g.adj[j]];
          if (lv < 0 || dist[lv] >= 0) continue;
          dist[lv] = dist[li] + 1;
          queue[qt++] = lv;
        }
      }
      start = last;
    }
    // grow side 0 in BFS order from the seed until it holds target0 weight;
    // disconnected remainders are entered from their lowest index.
    std::fill(cur.begin(), cur.end(), 1);
    std::fill(dist.begin(), dist.end(), -1);
    int64_t w0 = 0;
    int32_t qh = 0, qt = 0, next_unvisited = 0;
    dist[start] = 0;
    queue[qt++] = start;
    while (w0 < target0) {
      if (qh == qt) {
        while (next_unvisited < nv && dist[next_unvisited] >= 0) next_unvisited++;
        if (next_unvisited >= nv) break;
        dist[next_unvisited] = 0;
        queue[qt++] = next_unvisited;
      }
      int32_t li = queue[qh++];
      cur[li] = 0;
      w0 += g.vw[verts[li]];
      int32_t u = verts[li];
      for (int64_t j = g.xadj[u]; j < g.xadj[u + 1]; j++) {
        int32_t lv = local[g.adj[j]];
        if (lv < 0 || dist[lv] >= 0) continue;
        dist[lv] = 1;
        queue[qt++] = lv;
      }
    }
    // 2-way refinement: move boundary vertices with positive gain while the
    // balance stays within 3% of the target.
    const int64_t tol = std::max<int64_t>(1, (int64_t)(0.03 * (double)total / 2));
    int64_t wside[2] = {w0, total - w0};
    const int64_t tgt[2] = {target0, total - target0};
    for (int pass = 0; pass < 8; pass++) {
      int moved = 0;
      for (int32_t li = 0; li < nv; li++) {
        int32_t u = verts[li];
        int32_t s = cur[li];
        int64_t in = 0, out = 0;
        for (int64_t j = g.xadj[u]; j < g.xadj[u + 1]; j++) {
          int32_t lv = local[g.adj[j]];
          if (lv < 0) continue;
          (cur[lv] == s ? in : out) += g.ew[j];
        }
        if (out == 0) continue;
        int64_t gain = out - in;
        int32_t o = 1 - s;
        bool ok_bal = wside[o] + g.vw[u] <= tgt[o] + tol && wside[s] - g.vw[u] >= tgt[s] - tol;
        bool improves_bal = wside[s] - tgt[s] > wside[o] - tgt[o] + g.vw[u];
        if ((gain > 0 && ok_bal) || (gain == 0 && improves_bal)) {
          cur[li] = o;
          wside[s] -= g.vw[u];
          wside[o] += g.vw[u];
          moved++;
        }
      }
      if (!moved) break;
    }
    int64_t cut = 0;
    for (int32_t li = 0; li < nv; li++) {
      int32_t u = verts[li];
      for (int64_t j = g.xadj[u]; j < g.xadj[u + 1]; j++) {
        int32_t lv = local[g.adj[j]];
        if (lv >= 0 && cur[lv] != cur[li]) cut += g.ew[j];
      }
    }
    int64_t imb = std::llabs(wside[0] - target0);
    cut += imb * 4;  // prefer balanced candidates
    if (cut < best_cut) {
      best_cut = cut;
      best_side = cur;
    }
  }
  side = best_side;
}

void recursive_bisect(const WGraph &g, const std::vector<int32_t> &verts, int32_t k,
                      int32_t first_part, std::vector<int32_t> &part, std::mt19937_64 &rng) {
  if (k == 1 || verts.empty()) {
    for (int32_t v : verts) part[v] = first_part;
    return;
  }
  int32_t k0 = k / 2;
  int64_t total = 0;
  for (int32_t v : verts) total += g.vw[v];
  int64_t target0 = (int64_t)((double)total * k0 / k + 0.5);
  std::vector<int32_t> side;
  bisect(g, verts, target0, side, rng, 6);
  std::vector<int32_t> a, b;
  for (size_t i = 0; i < verts.size(); i++) (side[i] == 0 ? a : b).push_back(verts[i]);
  recursive_bisect(g, a, k0, first_part, part, rng);
  recursive_bisect(g, b, k - k0, first_part + k0, part, rng);
}

// Greedy K-way boundary refinement (move to the neighbouring part with the
// largest positive gain if the balance bound allows; zero-gain moves only if
// they improve the balance).
void kway_refine(const WGraph &g, std::vector<int32_t> &part, int32_t K, int64_t maxw,
                 std::mt19937_64 &rng, int passes) {
  std::vector<int64_t> pw(K, 0);
  for (int32_t u = 0; u < g.n; u++) pw[part[u]] += g.vw[u];
  std::vector<int64_t> conn(K, 0);
  std::vector<int32_t> touched;
  std::vector<int32_t> order(g.n);
  std::iota(order.begin(), order.end(), 0);
  for (int pass = 0; pass < passes; pass++) {
    std::shuffle(order.begin(), order.end(), rng);
    int moved = 0;
    for (int32_t u : order) {
      int32_t s = part[u];
      touched.clear();
      for (int64_t j = g.xadj[u]; j < g.xadj[u + 1]; j++) {
        int32_t p = part[g.adj[j]];
        if (conn[p] == 0) touched.push_back(p);
        conn[p] += g.ew[j];
      }
      int64_t in = conn[s];
      int32_t best = -1;
      int64_t best_gain = INT64_MIN;
      for (int32_t p : touched) {
        if (p == s) continue;
        int64_t gain = conn[p] - in;
        bool fits = pw[p] + g.vw[u] <= maxw;
        if (!fits) continue;
        if (gain > best_gain || (gain == best_gain && pw[p] < pw[best])) {
          best_gain = gain;
          best = p;
        }
      }
      for (int32_t p : touched) conn[p] = 0;
      if (best < 0) continue;
      bool overweight = pw[s] > maxw;
      if (best_gain > 0 || (best_gain == 0 && pw[best] + g.vw[u] < pw[s]) || overweight) {
        part[u] = best;
        pw[s] -= g.vw[u];
        pw[best] += g.vw[u];
        moved++;
      }
    }
    if (!moved) break;
  }
}

}  // namespace

int partition(int32_t n, const int32_t *ro, const int32_t *col, int32_t K, uint64_t seed,
              int32_t *graph_id, int64_t *edge_cut) {
  if (n < 0 || K < 1) return set_error(FAP_ERR_INVALID, "partition: need n >= 0 and K >= 1");
  std::mt19937_64 rng(seed ? seed : 1);
  std::vector<int32_t> part(n, 0);
  if (K > 1 && n > 0) {
    std::vector<WGraph> levels;
    std::vector<std::vector<int32_t>> maps;
    levels.push_back(symmetrize(n, ro, col));
    const int64_t coarse_target = std::max<int64_t>(40LL * K, 200);
    const int64_t max_vw = std::max<int64_t>(1, (int64_t)(1.5 * n / coarse_target));
    while (levels.back().n > coarse_target && levels.size() < 40) {
      std::vector<int32_t> cmap;
      WGraph c = coarsen(levels.back(), cmap, rng, max_vw);
      if (c.n > 0.95 * levels.back().n) break;
      maps.push_back(std::move(cmap));
      levels.push_back(std::move(c));
    }
    const WGraph &coarse = levels.back();
    std::vector<int32_t> cpart(coarse.n, 0);
    std::vector<int32_t> all(coarse.n);
    std::iota(all.begin(), all.end(), 0);
    recursive_bisect(coarse, all, K, 0, cpart, rng);
    const int64_t maxw = (int64_t)std::ceil(1.03 * (double)n / K);
    kway_refine(coarse, cpart, K, maxw, rng, 10);
    for (int lvl = (int)levels.size() - 2; lvl >= 0; lvl--) {
      std::vector<int32_t> fpart(levels[lvl].n);
      for (int32_t u = 0; u < levels[lvl].n; u++) fpart[u] = cpart[maps[lvl][u]];
      kway_refine(levels[lvl], fpart, K, maxw, rng, 6);
      cpart.swap(fpart);
    }
    part.swap(cpart);
  }
  int64_t cut = 0;
  for (int32_t u = 0; u < n; u++)
    for (int32_t j = ro[u]; j < ro[u + 1]; j++)
      if (col[j] > u && part[col[j]] != part[u]) cut++;
  for (int32_t u = 0; u < n; u++) graph_id[u] = part[u] + 1;
  if (edge_cut) *edge_cut = cut;
  return FAP_OK;
}

// ---------------------------------------------------------------------------
// Boundary marks and vertex order: findBoundry + sort_and_encode
// (fap/utils/util_preprocess.h:32-106).  The sort uses the reference's element
// layout and ordering rule with std::sort on the same input sequence, so the
// mapping (getMapping, fap/fap.cpp:546) is identical to the reference's.
// ---------------------------------------------------------------------------
namespace {
struct OrderKey {
  int v;
  int part;
  int bound;
};
bool order_before(const OrderKey &a, const OrderKey &b) {
  if (a.part == b.part) return a.bound > b.bound;
  return a.part < b.part;
}
}  // namespace

int preprocess(int32_t K, int32_t n, const int32_t *graph_id, const int32_t *ro,
               const int32_t *col, int32_t *st2ed, int32_t *ed2st, int32_t *ver_num,
               int32_t *ver_offset, int32_t *bdy_num, int32_t *bdy_offset,
               std::vector<uint8_t> *is_boundary) {
  if (K < 1 || n < 0) return set_error(FAP_ERR_INVALID, "preprocess: bad K or n");
  std::vector<uint8_t> isb(n, 0);
  std::vector<int32_t> cv(K + 1, 0), cb(K + 1, 0);
  for (int32_t u = 0; u < n; u++) {
    int32_t p = graph_id[u];
    if (p < 1 || p > K) return set_error(FAP_ERR_INVALID, "preprocess: part id outside 1..K");
    cv[p]++;
    for (int32_t j = ro[u]; j < ro[u + 1]; j++) {
      int32_t v = col[j];
      if (v < 0 || v >= n) return set_error(FAP_ERR_INVALID, "preprocess: column id out of range");
      if (graph_id[v] != p) {
        isb[u] = 1;
        isb[v] = 1;
      }
    }
  }
  for (int32_t u = 0; u < n; u++)
    if (isb[u]) cb[graph_id[u]]++;
  std::vector<OrderKey> keys(n);
  for (int32_t i = 0; i < n; i++) keys[i] = OrderKey{i, graph_id[i], (int)isb[i]};
  std::vector<OrderKey> sorted(keys);
  std::sort(sorted.begin(), sorted.end(), order_before);
  for (int32_t i = 0; i < n; i++) {
    st2ed[i] = sorted[i].v;
    ed2st[sorted[i].v] = i;
  }
  int32_t acc = 0;
  ver_num[0] = ver_offset[0] = bdy_num[0] = bdy_offset[0] = 0;
  for (int32_t i = 1; i <= K; i++) {
    ver_offset[i] = acc;
    ver_num[i] = cv[i];
    bdy_offset[i] = acc;
    bdy_num[i] = cb[i];
    acc += cv[i];
  }
  if (is_boundary) is_boundary->swap(isb);
  return FAP_OK;
}

}  // namespace fapi
