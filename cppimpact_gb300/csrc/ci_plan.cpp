// ci_plan.cpp -- see ci_plan.h.
#include "ci_plan.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

namespace ci {

// 3D Hilbert index after J. Skilling, "Programming the Hilbert curve", AIP Conf.
// Proc. 707 (2004): axes -> transposed Hilbert integer, then bit interleave.
uint64_t hilbert_key3(uint32_t x, uint32_t y, uint32_t z, int bits) {
  uint32_t X[3] = {x, y, z};
  const uint32_t M = 1u << (bits - 1);
  for (uint32_t Q = M; Q > 1; Q >>= 1) {
    const uint32_t P = Q - 1;
    for (int i = 0; i < 3; i++) {
      if (X[i] & Q) {
        X[0] ^= P;
      } else {
        const uint32_t t = (X[0] ^ X[i]) & P;
        X[0] ^= t;
        X[i] ^= t;
      }
    }
  }
  X[1] ^= X[0];
  X[2] ^= X[1];
  uint32_t t = 0;
  for (uint32_t Q = M; Q > 1; Q >>= 1)
    if (X[2] & Q) t ^= Q - 1;
  for (int i = 0; i < 3; i++) X[i] ^= t;
  uint64_t key = 0;
  for (int b = bits - 1; b >= 0; b--)
    for (int i = 0; i < 3; i++) key = (key << 1) | ((X[i] >> b) & 1u);
  return key;
}

bool build_plan(int N, int E, int npe, const double* xloc, const int* conn, int chunk_elements,
                int chunk_nodes, int target_ctas, Plan* plan, std::string* err) {
  Plan& P = *plan;
  P = Plan();
  P.N = N;
  P.E = E;
  P.npe = npe;
  if (N <= 0 || E <= 0 || (npe != 4 && npe != 10)) {
    *err = "mesh must have nodes, elements and 4 or 10 nodes per element";
    return false;
  }
  for (long long i = 0; i < (long long)E * npe; i++)
    if (conn[i] < 0 || conn[i] >= N) {
      *err = "element_nodes holds a node id outside [0, num_nodes)";
      return false;
    }

  // -- 1. Hilbert order of element centroids (vertex average) ------------------------
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int i = 0; i < N; i++)
    for (int k = 0; k < 3; k++) {
      lo[k] = std::min(lo[k], xloc[3 * i + k]);
      hi[k] = std::max(hi[k], xloc[3 * i + k]);
    }
  double ext = 0.0;
  for (int k = 0; k < 3; k++) ext = std::max(ext, hi[k] - lo[k]);
  if (!(ext > 0.0)) ext = 1.0;
  const int bits = 20;
  const double scale = ((1u << bits) - 1) / ext;
  std::vector<uint64_t> key(E);
  for (int e = 0; e < E; e++) {
    double c[3] = {0, 0, 0};
    for (int a = 0; a < 4; a++)
      for (int k = 0; k < 3; k++) c[k] += 0.25 * xloc[3 * (size_t)conn[(size_t)npe * e + a] + k];
    uint32_t q[3];
    for (int k = 0; k < 3; k++) q[k] = (uint32_t)std::llround((c[k] - lo[k]) * scale);
    key[e] = hilbert_key3(q[0], q[1], q[2], bits);
  }
  std::vector<int> sfc(E);
  std::iota(sfc.begin(), sfc.end(), 0);
  std::stable_sort(sfc.begin(), sfc.end(), [&](int a, int b) { return key[a] < key[b]; });

  // -- 2. chunks: contiguous runs along the curve bounded by elements and local nodes
  if (target_ctas <= 0) target_ctas = kDefaultTargetCtas;
  int emax = chunk_elements > 0 ? chunk_elements
                                : std::max(16, std::min(4096, (E + target_ctas - 1) / target_ctas));
  int lmax = chunk_nodes > 0 ? chunk_nodes : 896;
  lmax = std::max(lmax, npe);
  std::vector<int> stamp(N, -1), owner(N, -1), touch(N, 0);
  std::vector<int> cbeg;  // chunk start in sfc order
  {
    int c = -1, ne = 0, nl = 0;
    for (int i = 0; i < E; i++) {
      const int* en = conn + (size_t)npe * sfc[i];
      int fresh = 0;
      if (c >= 0)
        for (int a = 0; a < npe; a++) fresh += stamp[en[a]] != c;
      if (c < 0 || ne + 1 > emax || nl + fresh > lmax) {
        c++;
        cbeg.push_back(i);
        ne = nl = 0;
        fresh = npe;  // all new to the fresh chunk (duplicates impossible in a valid tet)
      }
      for (int a = 0; a < npe; a++)
        if (stamp[en[a]] != c) {
          stamp[en[a]] = c;
          nl++;
          touch[en[a]]++;
          if (owner[en[a]] < 0) owner[en[a]] = c;
        }
      ne++;
    }
    cbeg.push_back(E);
  }
  const int C = (int)cbeg.size() - 1;
  P.n_chunks = C;
  P.chunks.resize(C);

  // -- 3. node renumbering: owned nodes contiguous per chunk, interior ones first,
  //       each group in first-touch order -----------------------------------------
  P.node_new.assign(N, -1);
  P.node_orig.assign(N, -1);
  int next = 0;
  for (int c = 0; c < C; c++) {
    P.chunks[c].own_begin = next;
    for (int pass = 0; pass < 2; pass++) {
      for (int i = cbeg[c]; i < cbeg[c + 1]; i++) {
        const int* en = conn + (size_t)npe * sfc[i];
        for (int a = 0; a < npe; a++) {
          const int n = en[a];
          if (owner[n] == c && P.node_new[n] < 0 && (pass == 0) == (touch[n] == 1)) {
            P.node_new[n] = next;
            P.node_orig[next] = n;
            next++;
          }
        }
      }
      if (pass == 0) P.chunks[c].n_int = next - P.chunks[c].own_begin;
    }
    P.chunks[c].n_own = next - P.chunks[c].own_begin;
  }
  if (next != N) {
    *err = "mesh has nodes that no element references";
    return false;
  }

  // -- 4. local numbering, slot counts ---------------------------------------------
  std::vector<int> local(N, -1);
  std::fill(stamp.begin(), stamp.end(), -1);
  std::vector<std::vector<int>> chunk_gids(C);
  std::vector<int> nslots(N, 0);
  for (int c = 0; c < C; c++) {
    ChunkInfo& ch = P.chunks[c];
    std::vector<int>& g = chunk_gids[c];
    g.resize(ch.n_own);
    for (int l = 0; l < ch.n_own; l++) g[l] = ch.own_begin + l;
    for (int i = cbeg[c]; i < cbeg[c + 1]; i++) {
      const int* en = conn + (size_t)npe * sfc[i];
      for (int a = 0; a < npe; a++) {
        const int gn = P.node_new[en[a]];
        if (owner[en[a]] != c && stamp[gn] != c) {
          stamp[gn] = c;
          g.push_back(gn);
        }
      }
    }
    ch.n_local = (int)g.size();
    P.n_ghosts += ch.n_local - ch.n_own;
    for (int gn : g) nslots[gn]++;
    P.max_local = std::max(P.max_local, ch.n_local);
  }
  P.slot_row.assign(N + 1, 0);
  for (int n = 0; n < N; n++) {
    P.slot_row[n + 1] = P.slot_row[n] + nslots[n];
    if (nslots[n] > 1) P.n_boundary++;
  }
  std::vector<int> cursor(P.slot_row.begin(), P.slot_row.end() - 1);
  int lbeg = 0;
  for (int c = 0; c < C; c++) {
    P.chunks[c].local_begin = lbeg;
    // interior nodes come first in the owned range and have one slot each, so their
    // slots are contiguous from here
    P.chunks[c].slot_begin = P.chunks[c].n_own > 0 ? P.slot_row[P.chunks[c].own_begin] : 0;
    for (int gn : chunk_gids[c]) {
      P.local_gid.push_back(gn);
      P.local_slot.push_back(cursor[gn]++);
      P.local_srow.push_back(P.slot_row[gn]);
      P.local_srow.push_back(P.slot_row[gn + 1]);
    }
    lbeg += P.chunks[c].n_local;
  }

  // -- 5. per-chunk greedy colouring, elements sorted by (colour, curve order) -------
  P.elem_orig.resize(E);
  P.color.resize(E);
  P.conn_local.resize((size_t)npe * E);
  std::vector<uint64_t> used_lo(N), used_hi(N);
  for (int c = 0; c < C; c++) {
    ChunkInfo& ch = P.chunks[c];
    ch.elem_begin = cbeg[c];
    ch.elem_end = cbeg[c + 1];
    P.max_chunk_elems = std::max(P.max_chunk_elems, ch.elem_end - ch.elem_begin);
    const std::vector<int>& g = chunk_gids[c];
    for (int l = 0; l < ch.n_local; l++) local[g[l]] = l;
    for (int gn : g) used_lo[gn] = used_hi[gn] = 0;
    const int ne = ch.elem_end - ch.elem_begin;
    std::vector<int> col(ne);
    for (int i = 0; i < ne; i++) {
      const int* en = conn + (size_t)npe * sfc[ch.elem_begin + i];
      uint64_t lo_m = 0, hi_m = 0;
      for (int a = 0; a < npe; a++) {
        lo_m |= used_lo[P.node_new[en[a]]];
        hi_m |= used_hi[P.node_new[en[a]]];
      }
      int k;
      if (~lo_m) {
        k = __builtin_ctzll(~lo_m);
      } else if (~hi_m) {
        k = 64 + __builtin_ctzll(~hi_m);
      } else {
        *err = "a chunk needs more than 128 colours";
        return false;
      }
      col[i] = k;
      for (int a = 0; a < npe; a++) {
        const int gn = P.node_new[en[a]];
        if (k < 64)
          used_lo[gn] |= 1ull << k;
        else
          used_hi[gn] |= 1ull << (k - 64);
      }
      P.max_colors = std::max(P.max_colors, k + 1);
    }
    std::vector<int> ord(ne);
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return col[a] < col[b]; });
    for (int i = 0; i < ne; i++) {
      const int pe = ch.elem_begin + i;
      const int oe = sfc[ch.elem_begin + ord[i]];
      P.elem_orig[pe] = oe;
      P.color[pe] = (uint8_t)col[ord[i]];
      for (int a = 0; a < npe; a++)
        P.conn_local[(size_t)a * E + pe] = (uint16_t)local[P.node_new[conn[(size_t)npe * oe + a]]];
    }
  }
  if (P.max_local > 65535) {
    *err = "chunk local node count exceeds 16-bit local ids";
    return false;
  }
  return true;
}

int flow_lists(const Plan& P, std::vector<int>* own_row, std::vector<int>* own_idx,
               std::vector<int>* touch_row, std::vector<int>* touch_idx) {
  const int C = P.n_chunks;
  std::vector<int> owner(P.N, -1);
  for (int c = 0; c < C; c++)
    for (int l = 0; l < P.chunks[c].n_own; l++) owner[P.chunks[c].own_begin + l] = c;
  std::vector<std::vector<int>> own(C), touch(C);
  for (int c = 0; c < C; c++) {
    const ChunkInfo& ch = P.chunks[c];
    for (int l = 0; l < ch.n_local; l++) {
      const int g = l < ch.n_own ? ch.own_begin + l : P.local_gid[ch.local_begin + l];
      own[c].push_back(owner[g]);
      touch[owner[g]].push_back(c);
    }
  }
  int longest = 0;
  auto csr = [&longest](std::vector<std::vector<int>>& lists, std::vector<int>* row,
                        std::vector<int>* idx) {
    row->assign(1, 0);
    idx->clear();
    for (auto& v : lists) {
      std::sort(v.begin(), v.end());
      v.erase(std::unique(v.begin(), v.end()), v.end());
      longest = std::max(longest, (int)v.size());
      idx->insert(idx->end(), v.begin(), v.end());
      row->push_back((int)idx->size());
    }
  };
  csr(own, own_row, own_idx);
  csr(touch, touch_row, touch_idx);
  return longest;
}

std::vector<int> flow_order(int C, const std::vector<int>& own_row, const std::vector<int>& own_idx) {
  // symmetric adjacency without self loops
  std::vector<std::vector<int>> adj(C);
  for (int c = 0; c < C; c++)
    for (int k = own_row[c]; k < own_row[c + 1]; k++) {
      const int o = own_idx[k];
      if (o == c) continue;
      adj[c].push_back(o);
      adj[o].push_back(c);
    }
  for (auto& v : adj) {
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
  }
  auto by_degree = [&adj](int a, int b) {
    return adj[a].size() != adj[b].size() ? adj[a].size() < adj[b].size() : a < b;
  };
  for (auto& v : adj) std::sort(v.begin(), v.end(), by_degree);
  std::vector<int> level(C, -1), order;
  order.reserve(C);
  std::vector<int> seen(C, 0), bfs;
  // breadth-first levels from s within its component; returns the last level's nodes
  auto levels = [&](int s, std::vector<int>* comp) {
    comp->assign(1, s);
    level[s] = 0;
    for (size_t h = 0; h < comp->size(); h++) {
      const int u = (*comp)[h];
      for (int w : adj[u])
        if (level[w] < 0) {
          level[w] = level[u] + 1;
          comp->push_back(w);
        }
    }
    const int last = level[comp->back()];
    std::vector<int> far;
    for (int u : *comp) {
      if (level[u] == last) far.push_back(u);
      level[u] = -1;
    }
    return std::make_pair(last, far);
  };
  std::vector<int> comp;
  for (int c0 = 0; c0 < C; c0++) {
    if (seen[c0]) continue;
    // pseudo-peripheral start (George and Liu): move to a lowest-degree node of the
    // farthest level while the eccentricity grows
    int s = c0;
    auto lv = levels(s, &comp);
    for (int it = 0; it < 8; it++) {
      const int cand = *std::min_element(lv.second.begin(), lv.second.end(), by_degree);
      auto lv2 = levels(cand, &comp);
      if (lv2.first <= lv.first) break;
      s = cand;
      lv = lv2;
    }
    // Cuthill-McKee from s
    const size_t begin = order.size();
    order.push_back(s);
    seen[s] = 1;
    for (size_t h = begin; h < order.size(); h++)
      for (int w : adj[order[h]])
        if (!seen[w]) {
          seen[w] = 1;
          order.push_back(w);
        }
    std::reverse(order.begin() + begin, order.end());
  }
  return order;
}

bool verify_plan(const Plan& P, const int* conn, std::string* err) {
  const int E = P.E, N = P.N, npe = P.npe;
  std::vector<int> seen(E, 0);
  for (int e = 0; e < E; e++) seen[P.elem_orig[e]]++;
  for (int e = 0; e < E; e++)
    if (seen[e] != 1) {
      *err = "element not covered exactly once";
      return false;
    }
  for (int n = 0; n < N; n++)
    if (P.node_new[P.node_orig[n]] != n) {
      *err = "node permutation is not a bijection";
      return false;
    }
  std::vector<int> slot_hits(P.slot_row[N], 0);
  for (int c = 0; c < P.n_chunks; c++) {
    const ChunkInfo& ch = P.chunks[c];
    for (int l = 0; l < ch.n_local; l++) {
      const int gn = P.local_gid[ch.local_begin + l];
      const int s = P.local_slot[ch.local_begin + l];
      if (l < ch.n_own && gn != ch.own_begin + l) {
        *err = "owned local node does not map to the owned range";
        return false;
      }
      if ((l < ch.n_int) != (P.slot_row[gn + 1] - P.slot_row[gn] == 1)) {
        *err = "interior/boundary split does not match the slot counts";
        return false;
      }
      if (l < ch.n_int && (s != ch.slot_begin + l || P.slot_row[gn] != ch.slot_begin + l)) {
        *err = "interior slots are not contiguous from the chunk's slot_begin";
        return false;
      }
      if (P.local_srow[2 * (size_t)(ch.local_begin + l)] != P.slot_row[gn] ||
          P.local_srow[2 * (size_t)(ch.local_begin + l) + 1] != P.slot_row[gn + 1]) {
        *err = "local slot range does not match the node's slot row";
        return false;
      }
      if (s < P.slot_row[gn] || s >= P.slot_row[gn + 1]) {
        *err = "slot outside its node's slot row";
        return false;
      }
      slot_hits[s]++;
    }
    // colours: conflict-free and non-decreasing
    std::vector<int> last_color(ch.n_local, -1);
    for (int e = ch.elem_begin; e < ch.elem_end; e++) {
      if (e > ch.elem_begin && P.color[e] < P.color[e - 1]) {
        *err = "colours not sorted within a chunk";
        return false;
      }
      for (int a = 0; a < npe; a++) {
        const int l = P.conn_local[(size_t)a * E + e];
        if (l >= ch.n_local) {
          *err = "local id out of range";
          return false;
        }
        if (last_color[l] == P.color[e]) {
          *err = "two elements of one colour share a node";
          return false;
        }
        last_color[l] = P.color[e];
        const int gn = P.local_gid[ch.local_begin + l];
        if (P.node_orig[gn] != conn[(size_t)npe * P.elem_orig[e] + a]) {
          *err = "local connectivity does not match the mesh";
          return false;
        }
      }
    }
  }
  for (size_t s = 0; s < slot_hits.size(); s++)
    if (slot_hits[s] != 1) {
      *err = "slot not written exactly once";
      return false;
    }
  // the task kernel's dependency lists: own(c) holds exactly the owners of c's local nodes
  // (so an element task waits for every node task whose records it reads), touch(o)
  // exactly the chunks whose own list holds o (so a node task waits for every element
  // task that writes one of its nodes' halo slots), and the task order is a permutation
  std::vector<int> own_row, own_idx, touch_row, touch_idx;
  flow_lists(P, &own_row, &own_idx, &touch_row, &touch_idx);
  const int C = P.n_chunks;
  std::vector<int> owner(P.N, -1);
  for (int c = 0; c < C; c++)
    for (int l = 0; l < P.chunks[c].n_own; l++) owner[P.chunks[c].own_begin + l] = c;
  std::vector<int> mark(C, -1);
  for (int c = 0; c < C; c++) {
    const ChunkInfo& ch = P.chunks[c];
    int expect = 0;
    for (int l = 0; l < ch.n_local; l++) {
      const int o = owner[P.local_gid[ch.local_begin + l]];
      if (o < 0 || o > c) {
        *err = "a node's owner is not the first chunk touching it";
        return false;
      }
      if (mark[o] != c) {
        mark[o] = c;
        expect++;
      }
    }
    if (own_row[c + 1] - own_row[c] != expect) {
      *err = "own list does not match the owners of the chunk's nodes";
      return false;
    }
    for (int k = own_row[c]; k < own_row[c + 1]; k++) {
      const int o = own_idx[k];
      if (mark[o] != c) {
        *err = "own list names a chunk owning none of the chunk's nodes";
        return false;
      }
      if (!std::binary_search(touch_idx.begin() + touch_row[o], touch_idx.begin() + touch_row[o + 1], c)) {
        *err = "touch list misses a chunk holding one of the owner's nodes";
        return false;
      }
    }
  }
  if (own_idx.size() != touch_idx.size()) {
    *err = "own and touch lists are not each other's transpose";
    return false;
  }
  std::vector<int> order = flow_order(C, own_row, own_idx);
  std::sort(order.begin(), order.end());
  for (int k = 0; k < C; k++)
    if (order[k] != k) {
      *err = "task order of the chunks is not a permutation";
      return false;
    }
  return true;
}

}  // namespace ci
