/*
 * kinc_cli.cpp -- the native host driver: `kinc-gb300 run <analytic> --arg value ...` with
 * KINC's analytic names (src/core/analyticfactory.cpp:49-55) and argument names and defaults
 * (src/core/similarity_input.cpp, exportcorrelationmatrix_input.cpp, extract_input.cpp,
 * rmt_input.cpp, importexpressionmatrix_input.cpp, exportexpressionmatrix_input.cpp,
 * importcorrelationmatrix_input.cpp).  It does what ACE's serial runner does for these
 * analytics, through the C ABI only: read the expression matrix, create the worker, run the
 * ordered block loop into the CCM/CMX files (include/kinc_pairwise_matrix.h), run the analytics
 * downstream of them, or convert text to and from the matrix files.
 */
#include "../../include/kinc_pairwise_matrix.h"
#include "../../include/kinc_rmt.h"
#include "../../include/kinc_sim.h"

#include <algorithm>
#include <cctype>
#include <cerrno>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <map>
#include <string>
#include <vector>

#include <unistd.h>

namespace {

struct Args
{
   std::map<std::string, std::string> kv;
   /* cleared when a numeric argument does not parse (the message is printed) */
   mutable bool ok {true};

   bool has(const std::string& k) const { return kv.count(k) > 0; }
   std::string str(const std::string& k, const std::string& d = "") const
   {
      auto it = kv.find(k);
      return it == kv.end() ? d : it->second;
   }
   /* a decimal number (inf and nan included) */
   double real(const std::string& k, double d) const
   {
      if ( !has(k) ) return d;
      const std::string v = str(k);
      char* end = nullptr;
      const double x = std::strtod(v.c_str(), &end);
      if ( v.empty() || *end != '\0' ) return bad(k, "a number"), d;
      return x;
   }
   long long integer(const std::string& k, long long d) const
   {
      if ( !has(k) ) return d;
      const std::string v = str(k);
      char* end = nullptr;
      errno = 0;
      const long long x = std::strtoll(v.c_str(), &end, 10);
      if ( v.empty() || *end != '\0' || errno == ERANGE ) return bad(k, "an integer"), d;
      return x;
   }
   int int32(const std::string& k, int d) const
   {
      const long long x = integer(k, d);
      if ( x < INT32_MIN || x > INT32_MAX ) return bad(k, "a 32-bit integer"), d;
      return (int)x;
   }

private:
   void bad(const std::string& k, const char* what) const
   {
      fprintf(stderr, "--%s takes %s, got %s\n", k.c_str(), what, str(k).c_str());
      ok = false;
   }
};

/* The arguments each analytic takes (its input class's command-line names, plus the shard
 * and file options of this program). */
const std::map<std::string, std::vector<std::string>> KEYS = {
   { "similarity", { "input", "ccm", "cmx", "clusmethod", "corrmethod", "minexpr", "minsamp", "minclus", "maxclus",
                     "crit", "preout", "postout", "mincorr", "maxcorr", "ksize", "semantics", "precision",
                     "rand", "first-block", "blocks", "world", "rank", "by-cost", "resume", "little-endian",
                     "autotune" } },
   { "export-cmx", { "ccm", "cmx", "output", "little-endian" } },
   { "extract", { "emx", "ccm", "cmx", "output", "graphml", "mincorr", "maxcorr", "names", "little-endian" } },
   { "rmt", { "input", "log", "tstart", "tstep", "tstop", "minpace", "maxpace", "bins", "little-endian" } },
   { "import-emx", { "input", "output", "nan", "samples", "transform", "names", "sample-names", "little-endian" } },
   { "export-emx", { "input", "output", "nan", "transform", "names", "sample-names", "little-endian" } },
   { "import-cmx", { "input", "ccm", "cmx", "genes", "maxclusters", "samples", "corrname", "little-endian" } },
   { "merge", { "output", "inputs", "little-endian" } },
};

const std::vector<std::string> BOOLEANS = { "preout", "postout", "little-endian", "by-cost", "resume", "autotune" };

bool is_bool(const std::string& k)
{
   for ( const auto& b : BOOLEANS )
      if ( b == k ) return true;
   return false;
}

int usage()
{
   fprintf(stderr,
           "usage: kinc-gb300 run similarity --input EMX [--ccm CCM] [--cmx CMX] [--clusmethod none|gmm|kmeans]\n"
           "           [--corrmethod pearson|spearman|both] [--minexpr F] [--minsamp N] [--minclus N] [--maxclus N]\n"
           "           [--crit BIC|ICL] [--preout [true|false]] [--postout [true|false]] [--mincorr F] [--maxcorr F]\n"
           "           [--ksize N] [--semantics reference|fixed] [--precision fp32|tf32|3xbf16|fp32tiled|fp16]\n"
           "           [--rand glibc|lcg] [--first-block N] [--blocks N | --world N --rank R [--by-cost]] [--resume]\n"
           "           [--autotune] [--little-endian]\n"
           "       kinc-gb300 run export-cmx --ccm CCM --cmx CMX --output TXT\n"
           "       kinc-gb300 run extract --emx EMX --ccm CCM --cmx CMX [--output TXT] [--graphml XML] [--mincorr F]\n"
           "           [--maxcorr F] [--names TXT]\n"
           "       kinc-gb300 run rmt --input CMX --log TXT [--tstart F] [--tstep F] [--tstop F] [--minpace N]\n"
           "           [--maxpace N] [--bins N]\n"
           "       kinc-gb300 run import-emx --input TXT --output EMX [--nan TOKEN] [--samples N] [--transform NAME]\n"
           "           [--names TXT] [--sample-names TXT]\n"
           "       kinc-gb300 run export-emx --input EMX --output TXT [--nan TOKEN] [--transform NAME] [--names TXT]\n"
           "           [--sample-names TXT]\n"
           "       kinc-gb300 run import-cmx --input TXT --ccm CCM --cmx CMX --genes N --maxclusters N --samples N\n"
           "           --corrname NAME\n"
           "       kinc-gb300 run merge --output CCM|CMX --inputs RANK0,RANK1,...\n"
           "  (every analytic takes --little-endian; --transform: none, \"natural logarithm\", \"logarithm base 2\",\n"
           "   \"logarithm base 10\")\n");
   return 2;
}

bool parse(int argc, char** argv, int first, Args& a, std::string& err)
{
   for ( int i = first; i < argc; ++i )
   {
      std::string k = argv[i];
      if ( k.rfind("--", 0) != 0 )
      {
         err = "unexpected argument " + k;
         return false;
      }
      k = k.substr(2);
      const bool next_is_value = i + 1 < argc && std::strncmp(argv[i + 1], "--", 2) != 0;
      if ( is_bool(k) )
      {
         if ( next_is_value )
         {
            std::string v = argv[++i];
            for ( auto& ch : v ) ch = (char)std::tolower((unsigned char)ch);
            if ( v != "true" && v != "false" && v != "1" && v != "0" )
            {
               err = "--" + k + " takes true or false";
               return false;
            }
            a.kv[k] = (v == "true" || v == "1") ? "1" : "0";
         }
         else
         {
            a.kv[k] = "1";
         }
         continue;
      }
      if ( !next_is_value )
      {
         err = "--" + k + " needs a value";
         return false;
      }
      a.kv[k] = argv[++i];
   }
   return true;
}

int choice(const std::string& v, const std::vector<std::string>& names, const char* what, bool& ok)
{
   for ( size_t i = 0; i < names.size(); ++i )
   {
      std::string x = v, y = names[i];
      for ( auto& ch : x ) ch = (char)std::tolower((unsigned char)ch);
      for ( auto& ch : y ) ch = (char)std::tolower((unsigned char)ch);
      if ( x == y ) return (int)i;
   }
   fprintf(stderr, "%s must be one of:", what);
   for ( const auto& n : names ) fprintf(stderr, " %s", n.c_str());
   fprintf(stderr, "\n");
   ok = false;
   return 0;
}

/* --resume: cut the files an interrupted run left back to their whole work blocks
 * (kinc_pm_resume_point), run the remaining blocks into part files and join them after the kept
 * items (kinc_pm_concat); a file not yet created takes the part file as it is. */
int resume_to_files(kinc_sim_ctx* ctx, const std::string* ccm, const std::string* cmx, int le, int32_t G,
                    long long first_block, long long blocks)
{
   const long long B = KINC_SIM_WORK_BLOCK_SIZE;
   const long long total = (long long)G * (G - 1) / 2;
   const long long all = (total + B - 1) / B;
   const long long end = blocks < 0 ? all : std::min(all, first_block + blocks);
   int64_t start = 0;
   int rc = kinc_pm_resume_point(ccm ? ccm->c_str() : nullptr, cmx ? cmx->c_str() : nullptr, le, first_block, &start);
   if ( rc != KINC_SIM_OK ) return rc;
   if ( start > end )
   {
      fprintf(stderr, "similarity: the files hold work blocks past block %lld\n", end);
      return KINC_SIM_EINVAL;
   }
   const std::string ccm_part = ccm ? *ccm + ".part" : "", cmx_part = cmx ? *cmx + ".part" : "";
   rc = kinc_sim_run_to_files_ex(ctx, ccm ? ccm_part.c_str() : nullptr, cmx ? cmx_part.c_str() : nullptr, le, start,
                                 end - start, 0);
   if ( rc != KINC_SIM_OK ) return rc;
   for ( const std::string* final : { ccm, cmx } )
   {
      if ( !final ) continue;
      const std::string part = *final + ".part", joined = *final + ".joined";
      if ( access(final->c_str(), F_OK) == 0 )
      {
         const char* ins[2] = { final->c_str(), part.c_str() };
         if ( (rc = kinc_pm_concat(joined.c_str(), ins, 2, le)) != KINC_SIM_OK ) return rc;
         if ( std::rename(joined.c_str(), final->c_str()) != 0 || std::remove(part.c_str()) != 0 )
         {
            fprintf(stderr, "similarity: cannot replace %s\n", final->c_str());
            return KINC_SIM_EIO;
         }
      }
      else if ( std::rename(part.c_str(), final->c_str()) != 0 )
      {
         fprintf(stderr, "similarity: cannot create %s\n", final->c_str());
         return KINC_SIM_EIO;
      }
   }
   return KINC_SIM_OK;
}

int run_similarity(const Args& a)
{
   if ( !a.has("input") || (!a.has("ccm") && !a.has("cmx")) )
   {
      fprintf(stderr, "similarity: --input and --ccm and/or --cmx are required\n");
      return 2;
   }
   kinc_sim_params p;
   kinc_sim_params_default(&p);
   bool ok = true;
   p.clus_method = choice(a.str("clusmethod", "none"), { "none", "gmm", "kmeans" }, "clusmethod", ok);
   p.corr_method = choice(a.str("corrmethod", "pearson"), { "pearson", "spearman", "both" }, "corrmethod", ok);
   p.criterion = choice(a.str("crit", "ICL"), { "BIC", "ICL" }, "crit", ok);
   p.semantics = choice(a.str("semantics", "reference"), { "reference", "fixed" }, "semantics", ok);
   p.precision = choice(a.str("precision", "fp32"), { "fp32", "tf32", "3xbf16", "fp32tiled", "fp16" }, "precision", ok);
   p.rand_mode = choice(a.str("rand", "glibc"), { "glibc", "lcg" }, "rand", ok);
   if ( !ok ) return 2;
   p.min_expr = (float)a.real("minexpr", p.min_expr);
   p.min_samples = a.int32("minsamp", 30);
   p.min_clusters = a.int32("minclus", 1);
   p.max_clusters = a.int32("maxclus", 5);
   p.pre_out = a.str("preout", "0") == "1";
   p.post_out = a.str("postout", "0") == "1";
   p.min_corr = (float)a.real("mincorr", 0.5);
   p.max_corr = (float)a.real("maxcorr", 1.0);
   p.ksize = a.int32("ksize", 4096);
   long long first_block = a.integer("first-block", 0), blocks = a.integer("blocks", -1);
   const int world = a.int32("world", 0), rank = a.int32("rank", 0);
   if ( !a.ok ) return 2;
   if ( (a.has("world") || a.has("rank") || a.has("by-cost")) && (a.has("first-block") || a.has("blocks")) )
   {
      fprintf(stderr, "similarity: give --world/--rank or --first-block/--blocks, not both\n");
      return 2;
   }
   if ( (a.has("rank") || a.has("by-cost")) && !a.has("world") )
   {
      fprintf(stderr, "similarity: --rank and --by-cost need --world\n");
      return 2;
   }
   if ( a.has("world") && (world < 1 || rank < 0 || rank >= world) )
   {
      fprintf(stderr, "similarity: rank %d outside a world of %d\n", rank, world);
      return 2;
   }
   const int le = a.str("little-endian", "0") == "1";
   int32_t G = 0, S = 0;
   if ( kinc_emx_read_header(a.str("input").c_str(), le, &G, &S) != KINC_SIM_OK )
   {
      fprintf(stderr, "similarity: %s\n", kinc_pm_last_error());
      return 1;
   }
   std::vector<float> gem((size_t)G * S);
   if ( kinc_emx_read(a.str("input").c_str(), le, gem.data(), (int64_t)gem.size()) != KINC_SIM_OK )
   {
      fprintf(stderr, "similarity: %s\n", kinc_pm_last_error());
      return 1;
   }
   if ( a.has("world") )
   {
      int64_t fb = 0, nb = 0;
      if ( kinc_shard_blocks(gem.data(), G, S, p.min_expr, world, rank, a.str("by-cost", "0") == "1", &fb, &nb)
           != KINC_SIM_OK )
      {
         fprintf(stderr, "similarity: cannot shard %d genes over %d ranks\n", G, world);
         return 2;
      }
      first_block = fb;
      blocks = nb;
   }
   kinc_sim_ctx* ctx = nullptr;
   int rc = kinc_sim_create(gem.data(), G, S, &p, &ctx);
   if ( rc != KINC_SIM_OK )
   {
      fprintf(stderr, "similarity: %s\n", kinc_sim_last_error(nullptr));
      return 1;
   }
   if ( a.str("autotune", "0") == "1" && p.precision == 0 )
   {
      /* launch shape timed on pairs from the middle of the matrix (or taken from the tuning cache) */
      const int64_t total = kinc_sim_total_pairs(ctx);
      const int64_t size = std::min<int64_t>(total, (int64_t)4 * 32 * 16 * 152);
      kinc_sim_launch chosen {};
      int32_t n = 0;
      rc = kinc_sim_autotune(ctx, total / 2 - size / 2, size, 1, &chosen, nullptr, 0, &n);
      if ( rc != KINC_SIM_OK )
      {
         fprintf(stderr, "similarity: %s\n", kinc_sim_last_error(ctx));
         kinc_sim_destroy(ctx);
         return 1;
      }
      fprintf(stderr, "similarity: launch shape %d warps per CTA, rounds %d, prefetch %d (%s)\n",
              chosen.warps_per_cta, chosen.rounds, chosen.prefetch, n ? "timed" : "cached");
   }
   const std::string ccm = a.str("ccm"), cmx = a.str("cmx");
   if ( a.str("resume", "0") == "1" )
      rc = resume_to_files(ctx, a.has("ccm") ? &ccm : nullptr, a.has("cmx") ? &cmx : nullptr, le, G, first_block,
                           blocks);
   else
      rc = kinc_sim_run_to_files_ex(ctx, a.has("ccm") ? ccm.c_str() : nullptr, a.has("cmx") ? cmx.c_str() : nullptr,
                                    le, first_block, blocks, 0);
   if ( rc != KINC_SIM_OK ) fprintf(stderr, "similarity: %s\n", kinc_pm_last_error());
   kinc_sim_destroy(ctx);
   return rc == KINC_SIM_OK ? 0 : 1;
}

int run_export(const Args& a)
{
   if ( !a.has("ccm") || !a.has("cmx") || !a.has("output") )
   {
      fprintf(stderr, "export-cmx: --ccm, --cmx and --output are required\n");
      return 2;
   }
   const int rc = kinc_pm_export_text(a.str("ccm").c_str(), a.str("cmx").c_str(), a.str("little-endian", "0") == "1",
                                      a.str("output").c_str());
   if ( rc != KINC_SIM_OK ) fprintf(stderr, "export-cmx: %s\n", kinc_pm_last_error());
   return rc == KINC_SIM_OK ? 0 : 1;
}

int run_extract(const Args& a)
{
   if ( !a.has("emx") || !a.has("ccm") || !a.has("cmx") || (!a.has("output") && !a.has("graphml")) )
   {
      fprintf(stderr, "extract: --emx, --ccm, --cmx and --output and/or --graphml are required\n");
      return 2;
   }
   const float min_corr = (float)a.real("mincorr", 0.85), max_corr = (float)a.real("maxcorr", 1.0);
   if ( !a.ok ) return 2;
   const int rc = kinc_pm_extract(a.str("emx").c_str(), a.str("ccm").c_str(), a.str("cmx").c_str(),
                                  a.has("names") ? a.str("names").c_str() : nullptr,
                                  a.str("little-endian", "0") == "1",
                                  min_corr, max_corr,
                                  a.has("output") ? a.str("output").c_str() : nullptr,
                                  a.has("graphml") ? a.str("graphml").c_str() : nullptr);
   if ( rc != KINC_SIM_OK ) fprintf(stderr, "extract: %s\n", kinc_pm_last_error());
   return rc == KINC_SIM_OK ? 0 : 1;
}

int run_rmt(const Args& a)
{
   if ( !a.has("input") || !a.has("log") )
   {
      fprintf(stderr, "rmt: --input and --log are required\n");
      return 2;
   }
   kinc_rmt_params p;
   kinc_rmt_params_default(&p);
   p.threshold_start = (float)a.real("tstart", p.threshold_start);
   p.threshold_step = (float)a.real("tstep", p.threshold_step);
   p.threshold_stop = (float)a.real("tstop", p.threshold_stop);
   p.min_unfolding_pace = a.int32("minpace", p.min_unfolding_pace);
   p.max_unfolding_pace = a.int32("maxpace", p.max_unfolding_pace);
   p.histogram_bin_size = a.int32("bins", p.histogram_bin_size);
   if ( !a.ok ) return 2;
   float t = 0.0f;
   const int rc = kinc_rmt_run(a.str("input").c_str(), a.str("little-endian", "0") == "1", &p, a.str("log").c_str(), &t);
   if ( rc != KINC_SIM_OK )
   {
      fprintf(stderr, "rmt: %s\n", kinc_rmt_last_error());
      return 1;
   }
   printf("threshold: %g\n", (double)t);
   return 0;
}

const std::vector<std::string> TRANSFORMS = { "none", "natural logarithm", "logarithm base 2", "logarithm base 10" };

const char* opt(const Args& a, const char* k)
{
   auto it = a.kv.find(k);
   return it == a.kv.end() ? nullptr : it->second.c_str();
}

int run_import_emx(const Args& a)
{
   if ( !a.has("input") || !a.has("output") )
   {
      fprintf(stderr, "import-emx: --input and --output are required\n");
      return 2;
   }
   bool ok = true;
   const int t = choice(a.str("transform", "none"), TRANSFORMS, "transform", ok);
   if ( !ok ) return 2;
   const int samples = a.int32("samples", 0);
   if ( !a.ok ) return 2;
   const int rc = kinc_emx_import_text(opt(a, "input"), opt(a, "nan"), samples, t,
                                       a.str("little-endian", "0") == "1", opt(a, "output"), opt(a, "names"),
                                       opt(a, "sample-names"));
   if ( rc != KINC_SIM_OK ) fprintf(stderr, "import-emx: %s\n", kinc_pm_last_error());
   return rc == KINC_SIM_OK ? 0 : 1;
}

int run_export_emx(const Args& a)
{
   if ( !a.has("input") || !a.has("output") )
   {
      fprintf(stderr, "export-emx: --input and --output are required\n");
      return 2;
   }
   bool ok = true;
   const int t = choice(a.str("transform", "none"), TRANSFORMS, "transform", ok);
   if ( !ok ) return 2;
   const int rc = kinc_emx_export_text(opt(a, "input"), a.str("little-endian", "0") == "1", opt(a, "names"),
                                       opt(a, "sample-names"), t, opt(a, "nan"), opt(a, "output"));
   if ( rc != KINC_SIM_OK ) fprintf(stderr, "export-emx: %s\n", kinc_pm_last_error());
   return rc == KINC_SIM_OK ? 0 : 1;
}

int run_import_cmx(const Args& a)
{
   for ( const char* k : { "input", "ccm", "cmx", "genes", "maxclusters", "samples" } )
      if ( !a.has(k) )
      {
         fprintf(stderr, "import-cmx: --input, --ccm, --cmx, --genes, --maxclusters, --samples and --corrname are "
                         "required\n");
         return 2;
      }
   /* the correlation's name is metadata in KINC; it is required there, and not stored in the files */
   if ( a.str("corrname").empty() )
   {
      fprintf(stderr, "import-cmx: Correlation name is required.\n");
      return 2;
   }
   const int genes = a.int32("genes", 0), maxk = a.int32("maxclusters", 0), samples = a.int32("samples", 0);
   if ( !a.ok ) return 2;
   const int rc = kinc_pm_import_text(opt(a, "input"), opt(a, "ccm"), opt(a, "cmx"), genes, maxk, samples,
                                      a.str("little-endian", "0") == "1");
   if ( rc != KINC_SIM_OK ) fprintf(stderr, "import-cmx: %s\n", kinc_pm_last_error());
   return rc == KINC_SIM_OK ? 0 : 1;
}

int run_merge(const Args& a)
{
   if ( !a.has("output") || !a.has("inputs") )
   {
      fprintf(stderr, "merge: --output and --inputs (comma-separated, in rank order) are required\n");
      return 2;
   }
   std::vector<std::string> ins;
   const std::string list = a.str("inputs");
   for ( size_t b = 0;; )
   {
      const size_t e = list.find(',', b);
      ins.push_back(list.substr(b, e == std::string::npos ? std::string::npos : e - b));
      if ( e == std::string::npos ) break;
      b = e + 1;
   }
   std::vector<const char*> ptrs;
   for ( const auto& p : ins ) ptrs.push_back(p.c_str());
   const int rc = kinc_pm_concat(a.str("output").c_str(), ptrs.data(), (int32_t)ptrs.size(),
                                 a.str("little-endian", "0") == "1");
   if ( rc != KINC_SIM_OK ) fprintf(stderr, "merge: %s\n", kinc_pm_last_error());
   return rc == KINC_SIM_OK ? 0 : 1;
}

}  // namespace

int main(int argc, char** argv)
{
   if ( argc < 3 || std::strcmp(argv[1], "run") != 0 ) return usage();
   Args a;
   std::string err;
   if ( !parse(argc, argv, 3, a, err) )
   {
      fprintf(stderr, "%s\n", err.c_str());
      return usage();
   }
   const std::string an = argv[2];
   const auto keys = KEYS.find(an);
   if ( keys == KEYS.end() )
   {
      fprintf(stderr, "unknown analytic %s\n", an.c_str());
      return usage();
   }
   for ( const auto& kv : a.kv )
   {
      bool known = false;
      for ( const auto& k : keys->second ) known = known || k == kv.first;
      if ( !known )
      {
         fprintf(stderr, "%s: unknown argument --%s\n", an.c_str(), kv.first.c_str());
         return 2;
      }
   }
   if ( an == "similarity" ) return run_similarity(a);
   if ( an == "export-cmx" ) return run_export(a);
   if ( an == "extract" ) return run_extract(a);
   if ( an == "rmt" ) return run_rmt(a);
   if ( an == "import-emx" ) return run_import_emx(a);
   if ( an == "export-emx" ) return run_export_emx(a);
   if ( an == "import-cmx" ) return run_import_cmx(a);
   if ( an == "merge" ) return run_merge(a);
   fprintf(stderr, "unknown analytic %s\n", an.c_str());
   return usage();
}
