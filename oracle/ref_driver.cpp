/*
 * TEST INFRASTRUCTURE ONLY.  Drives KINC's own CPU Pairwise:: models
 * (compiled unmodified from the KINC source tree by oracle/build_ref.py) the
 * way Similarity::Serial does, so the C restatement in kinc_oracle.c and the
 * golden fixtures can be checked against the reference code itself.
 *
 * Restated here (the originals need the ACE framework):
 *   Similarity::Serial::execute    src/core/similarity_serial.cpp:33-101
 *   Similarity::Serial::fetchPair  src/core/similarity_serial.cpp:108-141
 *   Pairwise::Index(qint64), ++    src/core/pairwise_index.cpp:32-57,85-94
 * The models are the reference's: Pairwise::GMM, Pairwise::KMeans,
 * Pairwise::Pearson, Pairwise::Spearman.  rand() is the C library's, reset
 * with srand(1) and advanced by `rand_skip` draws, which puts it where a
 * fresh serial KINC process would be at the block start.  A call may span
 * several work blocks; the workspaces are renewed at each block boundary as
 * they are when ACE calls Serial::execute once per block.
 */
#include "pairwise_gmm.h"
#include "pairwise_kmeans.h"
#include "pairwise_pearson.h"
#include "pairwise_spearman.h"

#include <cmath>
#include <cstdint>
#include <cstdlib>

namespace {

int fetchPair(const float* gem, int S, int x, int y, float minExpression,
              QVector<Pairwise::Vector2>& X, QVector<qint8>& labels)
{
   const float* gene1 = gem + (int64_t)x * S;
   const float* gene2 = gem + (int64_t)y * S;
   int numSamples = 0;
   for ( int i = 0; i < S; ++i )
   {
      if ( std::isnan(gene1[i]) || std::isnan(gene2[i]) )
      {
         labels[i] = -9;
      }
      else if ( gene1[i] < minExpression || gene2[i] < minExpression )
      {
         labels[i] = -6;
      }
      else
      {
         X[numSamples] = { gene1[i], gene2[i] };
         numSamples++;
         labels[i] = 0;
      }
   }
   return numSamples;
}

void decode(int64_t index, int& x, int& y)
{
   int64_t xx = 1;
   int64_t pos = 0;
   while ( pos <= index )
   {
      ++xx;
      pos = xx * (xx - 1) / 2;
   }
   --xx;
   pos = xx * (xx - 1) / 2;
   x = (int)xx;
   y = (int)(index - pos);
}

}

extern "C" int kinc_ref_run_block(const float* gem, int G, int S, int clus_method, int corr_method,
                                  float min_expr, int min_samples, int min_clusters, int max_clusters,
                                  int criterion, int pre_out, int post_out, int64_t start, int64_t size,
                                  uint64_t rand_skip, int8_t* out_K, int8_t* out_labels, float* out_corr,
                                  int32_t* out_N)
{
   (void)G;
   ExpressionMatrix emx { S };
   Pairwise::Clustering* clus = nullptr;
   Pairwise::GMM gmm;
   Pairwise::KMeans kmeans;
   if ( clus_method == 1 )
   {
      clus = &gmm;
   }
   else if ( clus_method == 2 )
   {
      clus = &kmeans;
   }
   Pairwise::Pearson pearson;
   Pairwise::Spearman spearman;
   Pairwise::Correlation* corr = corr_method == 0 ? (Pairwise::Correlation*)&pearson
                                                  : (Pairwise::Correlation*)&spearman;
   if ( clus )
   {
      clus->initialize(&emx);
   }
   corr->initialize(&emx);

   srand(1);
   for ( uint64_t i = 0; i < rand_skip; ++i )
   {
      (void)rand();
   }

   QVector<Pairwise::Vector2> X(S);
   QVector<qint8> labels(S);
   int x, y;
   decode(start, x, y);
   for ( int64_t q = 0; q < size; ++q )
   {
      if ( q > 0 && (start + q) % 32768 == 0 )
      {
         /* Similarity::Serial::execute runs once per work block with fresh workspaces */
         X = QVector<Pairwise::Vector2>(S);
         labels = QVector<qint8>(S);
      }
      int numSamples = fetchPair(gem, S, x, y, min_expr, X, labels);
      qint8 K { 1 };
      if ( clus )
      {
         K = clus->compute(X, numSamples, labels, min_samples, (qint8)min_clusters, (qint8)max_clusters,
                           criterion == 0 ? Pairwise::Criterion::BIC : Pairwise::Criterion::ICL,
                           pre_out != 0, post_out != 0);
      }
      QVector<float> correlations = corr->compute(X, K, labels, min_samples);
      if ( out_K )
      {
         out_K[q] = K;
      }
      if ( out_labels )
      {
         for ( int i = 0; i < S; ++i )
         {
            out_labels[q * S + i] = labels[i];
         }
      }
      if ( out_corr )
      {
         for ( int k = 0; k < max_clusters; ++k )
         {
            out_corr[q * max_clusters + k] = k < K ? correlations[k] : NAN;
         }
      }
      if ( out_N )
      {
         out_N[q] = numSamples;
      }
      if ( ++y >= x )
      {
         y = 0;
         ++x;
      }
   }
   return 0;
}
