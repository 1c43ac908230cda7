// Layout checks of the cluster LDL^T's workspace and shared memory, run on
// the host (no device call): for every system size the cluster path takes
// (1..384 unknowns) and every cluster size, the workspace tiles and the push
// targets are 16-byte aligned, the mbarriers 8-byte aligned, the flag array
// lies past everything the chain CTA uses, the workspace fits the buffer
// the solver provides (chol_cluster_ws_doubles), and everything fits the
// largest opt-in shared memory of the part (227 KB).  Built and run by
// tests/test_chol_layout.py.
#include "mcba_chol.cu"

#include <cstdio>

int main() {
  using namespace mcba;
  int bad = 0;
  auto fail = [&](const char* what, int n, int C) {
    std::printf("FAIL %s: n=%d C=%d\n", what, n, C);
    ++bad;
  };
  const size_t max_smem = 227 * 1024, reserve = 1024;
  for (int n = 1; n <= kMaxBlk * kB; ++n) {
    const int nblk = (n + kB - 1) / kB;
    const int ld = 32 * ((n + 31) / 32);
    for (int C : {16, 8, 4}) {
      const Geo g = make_geo(C, ld, n);
      if (g.ws_doubles() > chol_cluster_ws_doubles(ld, n)) fail("workspace exceeds the solver's buffer", n, C);
      if (g.tile_off(1, 0) % 2 || g.m_offset() % 2 || g.p_offset() % 2) fail("workspace tile not 16-byte aligned", n, C);
      if (g.c_p(0) % 2 || g.c_diag(1) % 2) fail("push target not 16-byte aligned", n, C);
      if (g.b_mlast() < g.b_fl() + (size_t)(2 + nblk + 1) / 2) fail("counters overlap the last M", n, C);
      if (g.c_rx(1) >= g.c_end()) fail("receive mbarriers past the chain region", n, C);
      if (g.f_base() < g.c_end() || g.f_base() < g.b_end()) fail("flags overlap the chain CTA's data", n, C);
      if (g.f_base() + ((size_t)g.flag_count() + 1) / 2 > g.total()) fail("flags past the allocation", n, C);
      if (g.w_end() > g.total()) fail("worker buffers past the allocation", n, C);
      if (g.abort_index() != g.flag_count() - 1 || g.inv_index(nblk - 1) >= g.abort_index())
        fail("flag indices", n, C);
      if (g.total() * sizeof(double) + reserve > max_smem) fail("shared memory exceeds 227 KB", n, C);
    }
  }
  std::printf(bad ? "%d failures\n" : "layout ok\n", bad);
  return bad ? 1 : 0;
}
