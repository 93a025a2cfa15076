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

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <map>
#include <string>
#include <vector>

namespace {

struct Args
{
   std::map<std::string, std::string> kv;

   bool has(const std::string& k) const { return kv.count(k) > 0; }
   std::string str(const std::string& k, const std::string& d = "") const
   {
      auto it = kv.find(k);
      return it == kv.end() ? d : it->second;
   }
};

const std::vector<std::string> BOOLEANS = { "preout", "postout", "little-endian" };

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
           "           [--ksize N] [--first-block N] [--blocks N] [--little-endian]\n"
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

int run_similarity(const Args& a)
{
   if ( !a.has("input") || (!a.has("ccm") && !a.has("cmx")) )
   {
      fprintf(stderr, "similarity: --input and --ccm and/or --cmx are required\n");
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
   kinc_sim_params p;
   kinc_sim_params_default(&p);
   bool ok = true;
   p.clus_method = choice(a.str("clusmethod", "none"), { "none", "gmm", "kmeans" }, "clusmethod", ok);
   p.corr_method = choice(a.str("corrmethod", "pearson"), { "pearson", "spearman", "both" }, "corrmethod", ok);
   p.criterion = choice(a.str("crit", "ICL"), { "BIC", "ICL" }, "crit", ok);
   p.semantics = choice(a.str("semantics", "reference"), { "reference", "fixed" }, "semantics", ok);
   p.precision = choice(a.str("precision", "fp32"), { "fp32", "tf32", "3xbf16" }, "precision", ok);
   if ( !ok ) return 2;
   if ( a.has("minexpr") ) p.min_expr = (float)std::strtod(a.str("minexpr").c_str(), nullptr);
   p.min_samples = std::atoi(a.str("minsamp", "30").c_str());
   p.min_clusters = std::atoi(a.str("minclus", "1").c_str());
   p.max_clusters = std::atoi(a.str("maxclus", "5").c_str());
   p.pre_out = a.str("preout", "0") == "1";
   p.post_out = a.str("postout", "0") == "1";
   p.min_corr = (float)std::strtod(a.str("mincorr", "0.5").c_str(), nullptr);
   p.max_corr = (float)std::strtod(a.str("maxcorr", "1").c_str(), nullptr);
   p.ksize = std::atoi(a.str("ksize", "4096").c_str());
   kinc_sim_ctx* ctx = nullptr;
   int rc = kinc_sim_create(gem.data(), G, S, &p, &ctx);
   if ( rc != KINC_SIM_OK )
   {
      fprintf(stderr, "similarity: %s\n", kinc_sim_last_error(nullptr));
      return 1;
   }
   rc = kinc_sim_run_to_files_ex(ctx, a.has("ccm") ? a.str("ccm").c_str() : nullptr,
                                 a.has("cmx") ? a.str("cmx").c_str() : nullptr, le,
                                 std::atoll(a.str("first-block", "0").c_str()),
                                 std::atoll(a.str("blocks", "-1").c_str()), 0);
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
   const int rc = kinc_pm_extract(a.str("emx").c_str(), a.str("ccm").c_str(), a.str("cmx").c_str(),
                                  a.has("names") ? a.str("names").c_str() : nullptr,
                                  a.str("little-endian", "0") == "1",
                                  (float)std::strtod(a.str("mincorr", "0.85").c_str(), nullptr),
                                  (float)std::strtod(a.str("maxcorr", "1").c_str(), nullptr),
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
   if ( a.has("tstart") ) p.threshold_start = (float)std::strtod(a.str("tstart").c_str(), nullptr);
   if ( a.has("tstep") ) p.threshold_step = (float)std::strtod(a.str("tstep").c_str(), nullptr);
   if ( a.has("tstop") ) p.threshold_stop = (float)std::strtod(a.str("tstop").c_str(), nullptr);
   if ( a.has("minpace") ) p.min_unfolding_pace = std::atoi(a.str("minpace").c_str());
   if ( a.has("maxpace") ) p.max_unfolding_pace = std::atoi(a.str("maxpace").c_str());
   if ( a.has("bins") ) p.histogram_bin_size = std::atoi(a.str("bins").c_str());
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
   const int rc = kinc_emx_import_text(opt(a, "input"), opt(a, "nan"), std::atoi(a.str("samples", "0").c_str()), t,
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
   const int rc = kinc_pm_import_text(opt(a, "input"), opt(a, "ccm"), opt(a, "cmx"), std::atoi(a.str("genes").c_str()),
                                      std::atoi(a.str("maxclusters").c_str()), std::atoi(a.str("samples").c_str()),
                                      a.str("little-endian", "0") == "1");
   if ( rc != KINC_SIM_OK ) fprintf(stderr, "import-cmx: %s\n", kinc_pm_last_error());
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
   if ( an == "similarity" ) return run_similarity(a);
   if ( an == "export-cmx" ) return run_export(a);
   if ( an == "extract" ) return run_extract(a);
   if ( an == "rmt" ) return run_rmt(a);
   if ( an == "import-emx" ) return run_import_emx(a);
   if ( an == "export-emx" ) return run_export_emx(a);
   if ( an == "import-cmx" ) return run_import_cmx(a);
   fprintf(stderr, "unknown analytic %s\n", an.c_str());
   return usage();
}
