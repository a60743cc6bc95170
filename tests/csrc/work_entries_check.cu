// Host check of the split-BF16 contraction's work entries (ozaki_size):
// every K' tile a row block may hold nonzero values in is covered by exactly
// one entry, no other tile is, and the per-row-block tables agree.  Runs on
// the CPU (ozaki_size is host code); linked against the library's objects.
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "ff_ozaki.cuh"

using namespace sigma;

static int check(int nb, int nc, int ng, int nf, const std::vector<int>* kend, int grid) {
  FfDev d{};
  d.nb = nb;
  d.nc = nc;
  d.ng = ng;
  d.nf = nf;
  OzakiPrep oz{};
  OzakiTables t;
  ozaki_size(oz, d, grid, kend ? kend->data() : nullptr, &t);
  const int rows = nf * ng, kt = oz.kt;
  if (oz.n_items != oz.n_entries * oz.n_col_blocks || (int)t.entries.size() != oz.n_entries) return 1;
  std::vector<std::vector<int>> cover(oz.n_row_blocks, std::vector<int>(2 * kt, 0));
  std::vector<std::vector<int>> piece_seen(oz.n_row_blocks);
  for (const int4& e : t.entries) {
    if (e.x < 0 || e.x >= oz.n_row_blocks || e.w <= 0 || e.z < 0 || e.z + e.w > 2 * kt) return 2;
    for (int k = e.z; k < e.z + e.w; ++k) cover[e.x][k]++;
    piece_seen[e.x].push_back(e.y);
  }
  for (int rb = 0; rb < oz.n_row_blocks; ++rb) {
    int k = 0;
    for (int r = rb * kOzRows; r < std::min(rows, rb * kOzRows + kOzRows); ++r)
      k = std::max(k, std::min(kend ? (*kend)[r] : nc, nc));
    const int kl = (k + kOzKTile - 1) / kOzKTile;
    if (t.kt_lim[rb] != kl) return 3;
    for (int tile = 0; tile < 2 * kt; ++tile) {
      const bool active = (tile < kl) || (tile >= kt && tile < kt + kl);
      if (cover[rb][tile] != (active ? 1 : 0)) return 4;
    }
    if ((int)piece_seen[rb].size() != t.pieces[rb] || t.pieces[rb] > oz.max_pieces) return 5;
    std::vector<int> seen(t.pieces[rb], 0);
    for (int p : piece_seen[rb]) {
      if (p < 0 || p >= t.pieces[rb] || seen[p]++) return 6;
    }
  }
  return 0;
}

int main() {
  std::mt19937 rng(1);
  int bad = 0, n = 0;
  // the production shapes: FF (one slab per frequency), the GPP factor slabs,
  // the half-sum triangle
  const int shapes[][4] = {{512, 16384, 820, 15}, {512, 32768, 1638, 3}, {512, 32768, 1638, 1}};
  for (const auto& s : shapes) {
    bad += check(s[0], s[1], s[2], s[3], nullptr, 152) != 0;
    std::vector<int> kend(s[2] * s[3]);
    for (int r = 0; r < (int)kend.size(); ++r) kend[r] = std::min(s[1], (r % s[2] + 1) * 20);
    bad += check(s[0], s[1], s[2], s[3], &kend, 152) != 0;
    n += 2;
  }
  for (int i = 0; i < 3000; ++i) {
    const int nb = 1 + rng() % 600, nc = 1 + rng() % 40000, ng = 1 + rng() % std::min(nc, 2000);
    const int nf = 1 + rng() % 4, grid = 1 + rng() % 300;
    std::vector<int> kend(nf * ng);
    for (int& k : kend) k = (rng() % 5 == 0) ? 0 : (int)(rng() % (nc + 1));
    const int r1 = check(nb, nc, ng, nf, nullptr, grid), r2 = check(nb, nc, ng, nf, &kend, grid);
    if (r1 || r2) {
      if (bad < 5) std::printf("nb %d nc %d ng %d nf %d grid %d: %d %d\n", nb, nc, ng, nf, grid, r1, r2);
      ++bad;
    }
    n += 2;
  }
  std::printf("checked %d layouts, %d bad\n", n, bad);
  return bad ? 1 : 0;
}
