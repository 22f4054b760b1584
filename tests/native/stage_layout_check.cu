// Host-side check of the shared-memory stage layouts of the staged binary32
// kernels (rt_step8.cuh, rt_step11.cuh), compiled from the same headers the
// kernels use.  For every shape it enumerates an item's bulk copies and
// checks: the bytes the stage's mbarrier expects equal the bytes copied (a
// mismatch leaves the barrier incomplete), every copy lands inside the
// stage, copies do not overlap, and destinations and sizes are multiples of
// 16 bytes (the bulk-copy rule).  Exit status 0 when every shape passes.
#include <cstdio>
#include <vector>
#include <algorithm>

#include "rt_step11.cuh"

using namespace rt;

static int check_ranges(std::vector<std::pair<long long, long long>>& r, long long limit, const char* what,
                        const int* n, int G) {
  std::sort(r.begin(), r.end());
  for (size_t k = 0; k < r.size(); k++) {
    if (r[k].first < 0 || r[k].second > limit) {
      std::printf("%s out of the stage: n=%d,%d,%d G=%d [%lld,%lld) limit %lld\n", what, n[0], n[1], n[2], G,
                  r[k].first, r[k].second, limit);
      return 1;
    }
    if (k && r[k - 1].second > r[k].first) {
      std::printf("%s copies overlap: n=%d,%d,%d G=%d\n", what, n[0], n[1], n[2], G);
      return 1;
    }
  }
  return 0;
}

int main() {
  int bad = 0, w3_shapes = 0, w6_shapes = 0;
  const int spatial[] = {4, 8, 12, 16, 20, 24, 28, 32, 40, 48, 64};
  const int zs[] = {1, 2, 3, 4, 5, 6, 8, 16, 24, 32};
  const int spec[] = {1, 2, 4};
  for (int nx : spatial)
    for (int ny : spatial)
      for (int nz : zs)
        for (int nk : spec)
          for (int nm : spec) {
            Dims d{};
            d.n[0] = nx; d.n[1] = ny; d.n[2] = nz; d.n[3] = nk; d.n[4] = 2; d.n[5] = nm;
            // ---- fully staged plane kernel ----
            {
              w3_shapes++;
              const long long limit = (long long)w3_stage_floats(d) * 4;
              unsigned long long tot = 0;
              std::vector<std::pair<long long, long long>> r;
              for (int lane = 0; lane < 30; lane++) {
                const W3Copy c = w3_copy(d, lane);
                if (!c.valid) continue;
                if ((c.dst * 4) % 16 || c.bytes % 16) {
                  std::printf("w3 copy %d misaligned: n=%d,%d\n", lane, nx, ny);
                  bad++;
                }
                tot += c.bytes;
                r.push_back({c.dst * 4, c.dst * 4 + (long long)c.bytes});
              }
              if (tot != w3_tx_bytes(d)) {
                std::printf("w3 expects %u bytes, copies %llu: n=%d,%d,%d,%d,2,%d\n", w3_tx_bytes(d), tot, nx, ny,
                            nz, nk, nm);
                bad++;
              }
              bad += check_ranges(r, limit, "w3", d.n, 0);
            }
            // ---- z-slice kernel (every axis z..m longer than one) ----
            if (nz < 2 || nk < 2 || nm < 2) continue;
            for (int G = 1; G <= RT_W6_MAXG && G <= nz; G++) {
              w6_shapes++;
              const W6Layout L = w6_layout(d, G);
              const long long limit = (long long)L.floats() * 4;
              unsigned long long tot = 0;
              std::vector<std::pair<long long, long long>> r;
              for (int j = 0; j < L.copies(); j++) {
                const W6Copy c = w6_copy(L, j);
                if (((long long)c.dst * 4) % 16 || c.bytes % 16) {
                  std::printf("w6 copy %d misaligned: n=%d,%d G=%d\n", j, nx, ny, G);
                  bad++;
                }
                tot += c.bytes;
                r.push_back({(long long)c.dst * 4, (long long)c.dst * 4 + c.bytes});
              }
              if (tot != w6_tx_bytes(L)) {
                std::printf("w6 expects %u bytes, copies %llu: n=%d,%d,%d G=%d\n", w6_tx_bytes(L), tot, nx, ny, nz,
                            G);
                bad++;
              }
              bad += check_ranges(r, limit, "w6", d.n, G);
            }
          }
  std::printf("stage layouts: %d plane-kernel shapes, %d z-slice shapes, %d failures\n", w3_shapes, w6_shapes, bad);
  return bad ? 1 : 0;
}
