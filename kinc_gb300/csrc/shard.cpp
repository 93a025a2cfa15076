/*
 * shard.cpp -- the static partition of the work blocks across processes (include/kinc_sim.h:
 * kinc_shard_blocks).  Host code only.
 *
 * Cost of a block: the sum over its pairs (x, y) of n_x * n_y / S.  Pairs are enumerated row by
 * row (x = 1, 2, ...; y = 0 .. x-1, pair index x(x-1)/2 + y), so each row's pairs fall into at
 * most a few consecutive blocks and each block's share of a row is n_x times a range sum of a
 * prefix over n_y: O(genes + blocks) work however many pairs there are.  The cut between rank r
 * and r+1 is the first block boundary whose running cost reaches r/world of the total.
 */
#include "../../include/kinc_sim.h"

#include <algorithm>
#include <cmath>
#include <vector>

namespace {

int64_t total_pairs(int64_t genes)
{
   return genes * (genes - 1) / 2;
}

}  // namespace

extern "C" int kinc_shard_blocks(const float* gem, int32_t genes, int32_t samples, float min_expr, int32_t world,
                                 int32_t rank, int32_t by_cost, int64_t* first_block, int64_t* nblocks)
{
   if ( genes < 2 || samples < 1 || world < 1 || rank < 0 || rank >= world || !first_block || !nblocks
        || (by_cost && !gem) )
      return KINC_SIM_EINVAL;
   const int64_t B = KINC_SIM_WORK_BLOCK_SIZE;
   const int64_t total = total_pairs(genes);
   const int64_t nb = (total + B - 1) / B;
   int64_t b0 = nb * rank / world, b1 = nb * (rank + 1) / world;
   if ( by_cost )
   {
      std::vector<double> n((size_t)genes), prefix((size_t)genes + 1, 0.0);
      for ( int32_t g = 0; g < genes; ++g )
      {
         const float* row = gem + (size_t)g * samples;
         int64_t c = 0;
         for ( int32_t s = 0; s < samples; ++s ) c += !std::isnan(row[s]) && !(row[s] < min_expr);
         n[(size_t)g] = (double)c;
         prefix[(size_t)g + 1] = prefix[(size_t)g] + (double)c;
      }
      std::vector<double> cost((size_t)nb, 0.0);
      for ( int64_t x = 1; x < genes; ++x )
      {
         const int64_t p0 = x * (x - 1) / 2;
         for ( int64_t y = 0; y < x; )
         {
            const int64_t b = (p0 + y) / B;
            const int64_t y_end = std::min<int64_t>(x, (b + 1) * B - p0);
            cost[(size_t)b] += n[(size_t)x] * (prefix[(size_t)y_end] - prefix[(size_t)y]) / (double)samples;
            y = y_end;
         }
      }
      std::vector<double> run((size_t)nb + 1, 0.0);
      for ( int64_t b = 0; b < nb; ++b ) run[(size_t)b + 1] = run[(size_t)b] + cost[(size_t)b];
      const double whole = run[(size_t)nb];
      if ( whole > 0 )
      {
         auto cut = [&](int64_t r) -> int64_t {
            if ( r <= 0 ) return 0;
            if ( r >= world ) return nb;
            const double target = whole * (double)r / (double)world;
            return (int64_t)(std::lower_bound(run.begin(), run.end(), target) - run.begin());
         };
         b0 = cut(rank);
         b1 = cut(rank + 1);
      }
   }
   b0 = std::min(b0, nb);
   b1 = std::max(b0, std::min(b1, nb));
   *first_block = b0;
   *nblocks = b1 - b0;
   return KINC_SIM_OK;
}
