// cdt_core_host.cpp -- host build of the constrained Delaunay stage's mesh
// operations (surface-remesher_gb300/csrc/cdt_core.cuh), run one after the
// other on the CPU, for tests/test_cdt_core.py.  The GPU runs the same
// functions in parallel rounds; this replays the algorithm sequentially:
// adjacency of a starting triangulation, every constraint point located by a
// walk and inserted (inside, on an edge, or outside the hull), Lawson flips,
// each segment recovered by flips, flips again.
//
// stdin:  V, then V lines "X Y R"; T, then T lines "a b c" (counter-clockwise,
//         any triangulation of the first F points); C, then C point indices
//         to insert in order; S, then S lines "a b".
// stdout: "ok T L" (L segments left to the one-at-a-time pass) then T lines
//         "a b c", or "error <code>".
// argv[1] == "rounds": the segments go through the GPU's claim rounds first.
#include <algorithm>
#include <cstdio>
#include <string>
#include <map>
#include <utility>
#include <vector>

#include "cdt_core.cuh"

using namespace cvtgb::cdt;

int main(int argc, char **argv) {
  const bool rounds = argc > 1 && std::string(argv[1]) == "rounds";
  int serial = 0;
  int V = 0;
  if (scanf("%d", &V) != 1) return 1;
  std::vector<i64> X(V), Y(V), R(V);
  for (int v = 0; v < V; ++v)
    if (scanf("%lld %lld %lld", &X[v], &Y[v], &R[v]) != 3) return 1;
  int T = 0;
  if (scanf("%d", &T) != 1) return 1;
  const int cap = 2 * V + 16;
  std::vector<int> tri(3 * (size_t)cap), nbr(3 * (size_t)cap, kNone), vt(V, 0);
  std::vector<unsigned> cons(cap, 0);
  for (int t = 0; t < T; ++t)
    if (scanf("%d %d %d", &tri[3 * t], &tri[3 * t + 1], &tri[3 * t + 2]) != 3) return 1;
  std::map<std::pair<int, int>, int> dir;
  for (int t = 0; t < T; ++t)
    for (int i = 0; i < 3; ++i) {
      dir[{tri[3 * t + nx3(i)], tri[3 * t + pv3(i)]}] = pack_nb(t, i);
      vt[tri[3 * t + i]] = t;
    }
  for (int t = 0; t < T; ++t)
    for (int i = 0; i < 3; ++i) {
      auto it = dir.find({tri[3 * t + pv3(i)], tri[3 * t + nx3(i)]});
      nbr[3 * t + i] = it == dir.end() ? kNone : it->second;
    }
  Mesh m{tri.data(), nbr.data(), cons.data(), vt.data(), X.data(), Y.data(), R.data()};
  auto flips = [&]() {
    for (int round = 0; round < 1000000; ++round) {
      bool any = false;
      for (int t = 0; t < T; ++t)
        for (int i = 0; i < 3; ++i)
          if (wants_flip(m, t, i)) {
            flip(m, t, i);
            any = true;
          }
      if (!any) return true;
    }
    return false;
  };
  if (!flips()) {
    printf("error flips\n");
    return 0;
  }
  int C = 0;
  if (scanf("%d", &C) != 1) return 1;
  int start = 0;
  for (int k = 0; k < C; ++k) {
    int p;
    if (scanf("%d", &p) != 1) return 1;
    int t, i;
    const int kind = locate(m, p, start, 1 << 20, &t, &i);
    if (kind == kLocIn) {
      split_in(m, t, p, T, T + 1);
      T += 2;
    } else if (kind == kLocEdge) {
      const int two = nbr[3 * t + i] >= 0;
      split_edge(m, t, i, p, T, T + 1);
      T += two ? 2 : 1;
    } else if (kind == kLocOut) {
      std::vector<int> et, ei, bt, bi;
      int ft = t, fi = i;
      for (;;) {
        int pt, pi;
        if (!hull_prev(m, ft, fi, 4096, &pt, &pi)) {
          printf("error hull\n");
          return 0;
        }
        if (orient(m, tri[3 * pt + nx3(pi)], tri[3 * pt + pv3(pi)], p) >= 0) break;
        ft = pt;
        fi = pi;
        bt.push_back(pt);
        bi.push_back(pi);
      }
      for (int q = (int)bt.size() - 1; q >= 0; --q) {
        et.push_back(bt[q]);
        ei.push_back(bi[q]);
      }
      et.push_back(t);
      ei.push_back(i);
      int lt = t, li = i;
      for (;;) {
        int nt, ni;
        if (!hull_next(m, lt, li, 4096, &nt, &ni)) {
          printf("error hull\n");
          return 0;
        }
        if (orient(m, tri[3 * nt + nx3(ni)], tri[3 * nt + pv3(ni)], p) >= 0) break;
        lt = nt;
        li = ni;
        et.push_back(nt);
        ei.push_back(ni);
      }
      std::vector<int> slots(et.size());
      for (size_t q = 0; q < et.size(); ++q) slots[q] = T + (int)q;
      insert_out(m, et.data(), ei.data(), (int)et.size(), p, slots.data());
      T += (int)et.size();
    } else {
      printf("error locate %d\n", kind);
      return 0;
    }
    start = vt[p];
    if (!flips()) {
      printf("error flips\n");
      return 0;
    }
  }
  int S = 0;
  if (scanf("%d", &S) != 1) return 1;
  std::vector<int> queue(2 * 4096), stack(2 * 256), sa(S), sb(S);
  for (int k = 0; k < S; ++k)
    if (scanf("%d %d", &sa[k], &sb[k]) != 2) return 1;
  // rounds: the GPU's parallel segment rounds replayed (cdt.cu k_seg_mark,
  // k_seg_locate, k_seg_apply); each winner's recovery must change only
  // triangles it claimed and vt only of vertices it claimed around, and no
  // two winners may share a claimed triangle
  std::vector<int> state(S, 0);  // 0 pending, 1 done, 2 left to the one-at-a-time pass
  if (rounds) {
    const int kCorr = 8, kClaim = 128;
    for (int k = 0; k < S; ++k) state[k] = mark_constraint(m, sa[k], sb[k], 4096) ? 1 : 0;
    for (int round = 0; round < 100000; ++round) {
      std::vector<unsigned> cl(T, 0xffffffffu);
      std::vector<std::vector<int>> lists(S), verts(S);
      for (int k = 0; k < S; ++k) {
        if (state[k] != 0) continue;
        int q[2 * kCorr], on = -1, cnt = 0;
        if (collect_crossings(m, sa[k], sb[k], q, kCorr, 1 << 20, &on, &cnt) != kSegOk) {
          state[k] = 2;
          continue;
        }
        std::vector<int> L(kClaim);
        int n = 0;
        bool ok = true;
        for (int e = -2; e < 2 * cnt && ok; ++e) {
          const int v = e == -2 ? sa[k] : (e == -1 ? sb[k] : q[e]);
          bool seen = false;
          for (int f = -2; f < e && !seen; ++f)
            seen = (f == -2 ? sa[k] : (f == -1 ? sb[k] : q[f])) == v;
          if (seen) continue;
          verts[k].push_back(v);
          const int c = fan(m, v, 4096, L.data() + n, kClaim - n);
          if (c < 0) ok = false;
          else n += c;
        }
        if (!ok) {
          state[k] = 2;
          continue;
        }
        L.resize(n);
        for (int t : L) cl[t] = std::min(cl[t], prio((unsigned)k));
        lists[k] = L;
      }
      bool any = false;
      std::vector<int> owner(T, -1);
      for (int k = 0; k < S; ++k) {
        if (state[k] != 0) continue;
        bool won = true;
        for (int t : lists[k]) won = won && cl[t] == prio((unsigned)k);
        if (!won) continue;
        for (int t : lists[k]) {
          if (owner[t] >= 0 && owner[t] != k) {
            printf("error shared claim\n");
            return 0;
          }
          owner[t] = k;
        }
        const std::vector<int> tri0(tri.begin(), tri.begin() + 3 * T),
            nbr0(nbr.begin(), nbr.begin() + 3 * T), vt0(vt);
        const std::vector<unsigned> cons0(cons.begin(), cons.begin() + T);
        int q[2 * kCorr], on = -1;
        const int r = recover_segment(m, sa[k], sb[k], q, kCorr, 1 << 20, &on);
        if (r != kSegOk) {
          printf("error segment %d\n", r);
          return 0;
        }
        for (int t = 0; t < T; ++t) {
          bool changed = cons[t] != cons0[t];
          for (int i = 0; i < 3; ++i)
            changed = changed || tri[3 * t + i] != tri0[3 * t + i] || nbr[3 * t + i] != nbr0[3 * t + i];
          if (changed && cl[t] != prio((unsigned)k)) {
            printf("error unclaimed write\n");
            return 0;
          }
        }
        for (int v = 0; v < V; ++v)
          if (vt[v] != vt0[v] &&
              std::find(verts[k].begin(), verts[k].end(), v) == verts[k].end()) {
            printf("error unclaimed vertex\n");
            return 0;
          }
        state[k] = 1;
        any = true;
      }
      if (!any) break;
    }
  }
  for (int k = 0; k < S; ++k) {
    if (state[k] == 1) continue;
    if (state[k] == 2) ++serial;
    const int r = recover_chain(m, sa[k], sb[k], queue.data(), 4096, stack.data(), 256, 1 << 20);
    if (r != kSegOk) {
      printf("error segment %d\n", r);
      return 0;
    }
  }
  if (!flips()) {
    printf("error flips\n");
    return 0;
  }
  // the GPU's output order: by owner (smallest vertex), then second vertex
  std::vector<int> cnt(V + 1, 0), off(V + 1, 0), out(3 * (size_t)T, -1);
  for (int t = 0; t < T; ++t) {
    int a, b, c;
    canon(&tri[3 * t], a, b, c);
    ++cnt[a];
  }
  for (int v = 0; v < V; ++v) off[v + 1] = off[v] + cnt[v];
  for (int t = 0; t < T; ++t) {
    int a, b, c;
    canon(&tri[3 * t], a, b, c);
    const int r = owner_rank(m, t, 4096);
    const int pos = off[a] + r;
    if (r < 0 || pos >= T || out[3 * pos] != -1) {
      printf("error emit\n");
      return 0;
    }
    out[3 * pos] = a;
    out[3 * pos + 1] = b;
    out[3 * pos + 2] = c;
  }
  printf("ok %d %d\n", T, serial);
  for (int t = 0; t < T; ++t) printf("%d %d %d\n", out[3 * t], out[3 * t + 1], out[3 * t + 2]);
  return 0;
}
