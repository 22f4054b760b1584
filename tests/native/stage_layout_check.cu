// Host-side check of the shared-memory stage layouts of the staged binary32
// kernels (rt_step8.cuh, rt_step11.cuh), compiled from the same headers the
// kernels use.  For every shape (and, for the z-slice kernel, every first
// slice of an item) it enumerates an item's bulk copies and checks: the
// bytes the stage's mbarrier expects equal the bytes copied (a mismatch
// leaves the barrier incomplete), every copy lands inside the stage, copies
// do not overlap, destinations and sizes are multiples of 16 bytes (the
// bulk-copy rule), and every shared-memory slot the consumers read for a
// live cell is written by a copy.  Exit status 0 when every shape passes.
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
              {
                const long long pb = (long long)nx * ny * 4;
                auto covered = [&](long long lo, long long hi) {
                  for (auto& q : r)
                    if (q.first <= lo && hi <= q.second) return true;
                  return false;
                };
                bool ok = covered(0, pb) && covered((long long)RT_W3_VX * pb, (RT_W3_VX + 1) * pb) &&
                          covered((long long)RT_W3_VY * pb, (RT_W3_VY + 1) * pb) &&
                          covered((long long)RT_W3_LAM * pb, (RT_W3_LAM + 1) * pb) &&
                          covered((long long)RT_W3_NPL * pb, RT_W3_NPL * pb + ny * 4LL) &&
                          covered(RT_W3_NPL * pb + ny * 4LL, RT_W3_NPL * pb + (nx + ny) * 4LL);
                for (int a = 2; a < 6; a++) {
                  if (d.n[a] < 2) continue;
                  for (int i = 0; i < 4; i++)
                    ok = ok && covered((1 + 4 * (a - 2) + i) * pb, (2 + 4 * (a - 2) + i) * pb);
                  ok = ok && covered((RT_W3_VR + a - 2) * pb, (RT_W3_VR + a - 1) * pb) &&
                       covered((RT_W3_VL + a - 2) * pb, (RT_W3_VL + a - 1) * pb);
                }
                if (!ok) {
                  std::printf("w3 plane read but not written: n=%d,%d,%d,%d,2,%d\n", nx, ny, nz, nk, nm);
                  bad++;
                }
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
              const W6Layout L = w6_layout(d, G);
              const long long limit = (long long)L.floats() * 4;
              for (int z0 = 0; z0 < nz; z0 += G) {
                w6_shapes++;
                unsigned long long tot = 0;
                std::vector<std::pair<long long, long long>> r;
                for (int j = 0; j < RT_W6_NCOPY; j++) {
                  const W6Copy c = w6_copy(L, j, z0, nz);
                  if (!c.valid) continue;
                  if (((long long)c.dst * 4) % 16 || c.bytes % 16 || c.bytes == 0) {
                    std::printf("w6 copy %d misaligned or empty: n=%d,%d G=%d z0=%d\n", j, nx, ny, G, z0);
                    bad++;
                  }
                  tot += c.bytes;
                  r.push_back({(long long)c.dst * 4, (long long)c.dst * 4 + c.bytes});
                }
                if (tot != w6_tx_bytes(L, z0, nz)) {
                  std::printf("w6 expects %u bytes, copies %llu\n", w6_tx_bytes(L, z0, nz), tot);
                  bad++;
                }
                bad += check_ranges(r, limit, "w6", d.n, G);
                // every slot a live slice reads is written by a copy
                auto covered = [&](long long lo, long long hi) {
                  for (auto& q : r)
                    if (q.first <= lo && hi <= q.second) return true;
                  return false;
                };
                const long long pb = (long long)L.P * 4;
                for (int g = 0; g < G && z0 + g < nz; g++) {
                  bool ok = true;
                  for (int zz = g; zz <= g + 4; zz++) ok = ok && covered((long long)L.ez(zz) * 4, L.ez(zz) * 4 + pb);
                  for (int a = 3; a < 6; a++)
                    for (int i = 0; i < 4; i++) ok = ok && covered((long long)L.en(g, a, i) * 4, L.en(g, a, i) * 4 + pb);
                  for (int k = 0; k < 11; k++) ok = ok && covered((long long)L.v(g, k) * 4, L.v(g, k) * 4 + pb);
                  ok = ok && covered((long long)L.b0x(g) * 4, (L.b0x(g) + ny) * 4LL);
                  ok = ok && covered((long long)L.b0y(g) * 4, (L.b0y(g) + nx) * 4LL);
                  if (!ok) {
                    std::printf("w6 slot of live slice %d not written: n=%d,%d,%d G=%d z0=%d\n", g, nx, ny, nz, G, z0);
                    bad++;
                    break;
                  }
                }
              }
            }
          }
  std::printf("stage layouts: %d plane-kernel shapes, %d z-slice shapes, %d failures\n", w3_shapes, w6_shapes, bad);
  return bad ? 1 : 0;
}
