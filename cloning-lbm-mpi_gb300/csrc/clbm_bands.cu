// clbm_bands.cu -- row splits of a lattice over the CTAs of a cluster (host).
//
// The cluster-resident interval kernel keeps band b of every clone (rows
// [row0[b], row0[b+1])) in the shared memory of cluster rank b, and every
// step of the interval ends at a cluster barrier, so a step lasts as long as
// the slowest band.  Nodes are not equally costly: the walls and the square's
// box take the general update path (bounce-back masks, drag terms), several
// times a bulk node, and a band's first and last rows read and write the
// neighbouring CTAs.  An even split leaves the band holding the square the
// slowest; a balanced split gives it fewer rows.  The split does not change
// the results: every node is updated by the same arithmetic in any band.
#include <algorithm>
#include <limits>
#include <vector>

#include "clbm_internal.h"

namespace clbm {

void even_band_rows(int H, int cs, int *row0) {
  const int base = H / cs, extra = H % cs;
  for (int b = 0; b <= cs; b++) row0[b] = b * base + std::min(b, extra);
}

// Per-step cost of row y in node units: W, plus gamma per node on the
// general path (in a row of the square's box, the 32-node segments,
// row-aligned, that touch the box) and gamma / 4 per node of a wall row
// (bounce-back built into the bulk update).
static double row_cost(int W, int H, int xmin, int xmax, int ymin, int ymax, int y, double gamma) {
  double g = 0.0;
  if (y == 0 || y == H - 1) {
    g = 0.25 * W;
  } else if (y >= ymin && y <= ymax) {
    const int x0 = std::max(0, xmin) / 32 * 32;
    const int x1 = std::min(W, (std::min(W - 1, xmax) / 32 + 1) * 32);
    g = std::max(0, x1 - x0);
  }
  return W + gamma * g;
}

// The split of H rows into cs bands of at most rows_limit rows that
// minimises the largest band cost (row costs, plus gamma / 4 per node of
// each band-edge row that has a neighbour band) and, among splits with that
// largest cost, the sum of squared band costs (the other bands evened out):
// dynamic programming over (bands, rows) on the pair compared in that order.
bool balanced_band_rows(int W, int H, int xmin, int xmax, int ymin, int ymax, int cs, double gamma,
                        int rows_limit, int *row0) {
  if (cs < 1 || H < cs || rows_limit < 1 || (long long)cs * rows_limit < H) return false;
  if (gamma <= 0.0) {
    even_band_rows(H, cs, row0);
    for (int b = 0; b < cs; b++)
      if (row0[b + 1] - row0[b] > rows_limit) return false;
    return true;
  }
  std::vector<double> pre(H + 1, 0.0);
  for (int y = 0; y < H; y++) pre[y + 1] = pre[y] + row_cost(W, H, xmin, xmax, ymin, ymax, y, gamma);
  const double edge = 0.25 * gamma * W;
  auto band = [&](int a, int b) { return pre[b] - pre[a] + (a > 0 ? edge : 0.0) + (b < H ? edge : 0.0); };
  const double inf = std::numeric_limits<double>::infinity();
  // best[j][y] / sq[j][y]: largest band cost and sum of squares of rows
  // [0, y) in j bands; from[j][y]: the last band's first row
  std::vector<std::vector<double>> best(cs + 1, std::vector<double>(H + 1, inf));
  std::vector<std::vector<double>> sq(cs + 1, std::vector<double>(H + 1, inf));
  std::vector<std::vector<int>> from(cs + 1, std::vector<int>(H + 1, -1));
  best[0][0] = 0.0;
  sq[0][0] = 0.0;
  for (int j = 1; j <= cs; j++)
    for (int y = j; y <= H; y++)
      for (int x = std::max(j - 1, y - rows_limit); x < y; x++) {
        if (best[j - 1][x] == inf) continue;
        const double cb = band(x, y);
        const double c = std::max(best[j - 1][x], cb), q = sq[j - 1][x] + cb * cb;
        if (c < best[j][y] || (c == best[j][y] && q < sq[j][y])) {
          best[j][y] = c;
          sq[j][y] = q;
          from[j][y] = x;
        }
      }
  if (best[cs][H] == inf) return false;
  row0[cs] = H;
  for (int j = cs, y = H; j >= 1; j--) {
    y = from[j][y];
    row0[j - 1] = y;
  }
  return row0[0] == 0;
}

}  // namespace clbm
