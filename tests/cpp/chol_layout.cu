// Layout checks of the cluster LDL^T's workspace and shared memory, run on
// the host (no device call): for every system size the cluster path takes
// (1..384 unknowns) and every backward-solve slot count, the bulk-copy
// targets and sources are 16-byte aligned, the mbarriers 8-byte aligned, the
// flag array lies past everything the chain CTA uses, the workspace fits
// the buffer the solver provides (chol_cluster_ws_doubles), and the slot
// count the plan
// picks for the largest opt-in shared memory of the part (227 KB) leaves at
// least three slots.  Built and run by tests/test_chol_layout.py.
#include "mcba_chol.cu"

#include <cstdio>

int main() {
  using namespace mcba;
  int bad = 0;
  auto fail = [&](const char* what, int n, int R) {
    std::printf("FAIL %s: n=%d R=%d\n", what, n, R);
    ++bad;
  };
  const size_t max_smem = 227 * 1024, reserve = 1024;
  for (int n = 1; n <= kMaxBlk * kB; ++n) {
    const int nblk = (n + kB - 1) / kB;
    const int ld = 32 * ((n + 31) / 32);
    for (int C : {16, 8, 4}) {
      for (int R = 1; R <= nblk; ++R) {
        const Geo g = make_geo(C, ld, n, R);
        if (g.ws_doubles() > chol_cluster_ws_doubles(ld, n)) fail("workspace exceeds the solver's buffer", n, R);
        if (g.tile_off(1, 0) % 2 || g.m_offset() % 2 || g.p_offset() % 2)
          fail("workspace tile not 16-byte aligned", n, R);
        for (int s = 0; s <= R; ++s)
          if (g.b_slot(s) % 2) fail("backward slot not 16-byte aligned", n, R);
        if (g.c_p(0) % 2 || g.c_diag(1) % 2) fail("push target not 16-byte aligned", n, R);
        if (g.b_bar() + (size_t)R > g.b_slot(0)) fail("slot mbarriers overlap slot 0", n, R);
        if (g.c_rx(1) >= g.c_end()) fail("receive mbarriers past the chain region", n, R);
        if (g.f_base() < g.c_end() || g.f_base() < g.b_end()) fail("flags overlap the chain CTA's data", n, R);
        if (g.f_base() + ((size_t)g.flag_count() + 1) / 2 > g.total()) fail("flags past the allocation", n, R);
        if (g.w_end() > g.total()) fail("worker buffers past the allocation", n, R);
        if (g.abort_index() != g.flag_count() - 1 || g.inv_index(nblk - 1) >= g.abort_index())
          fail("flag indices", n, R);
      }
      // the plan's slot count for this size (largest that fits, at least min(nblk, 3))
      int R = nblk;
      while (R > (nblk < 3 ? nblk : 3) && make_geo(C, ld, n, R).total() * sizeof(double) + reserve > max_smem) --R;
      if (make_geo(C, ld, n, R).total() * sizeof(double) + reserve > max_smem) fail("no slot count fits", n, R);
    }
  }
  std::printf(bad ? "%d failures\n" : "layout ok\n", bad);
  return bad ? 1 : 0;
}
