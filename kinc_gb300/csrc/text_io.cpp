/*
 * text_io.cpp -- the text analytics on either side of the matrix files
 * (include/kinc_pairwise_matrix.h):
 *   ImportExpressionMatrix  text -> EMX        src/core/importexpressionmatrix.cpp:20-180
 *   ExportExpressionMatrix  EMX -> text        src/core/exportexpressionmatrix.cpp:20-100
 *   ImportCorrelationMatrix text -> CCM + CMX  src/core/importcorrelationmatrix.cpp:22-141
 *
 * KINC reads text through Qt's text stream: each line split on white space, numbers parsed by
 * QString::toInt / toFloat / toDouble in the C locale (a float is the double rounded to float),
 * numbers written at a fixed count of significant digits.  Here lines are split on ASCII white
 * space and numbers parsed with std::from_chars, which is locale-independent and correctly
 * rounded like Qt's parser.  Host code only.
 */
#include "../../include/kinc_pairwise_matrix.h"
#include "sim_internal.h"

#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <string_view>
#include <vector>

namespace {

/* getline(3) over a FILE*, with the buffer owned here. */
class Lines
{
public:
   explicit Lines(FILE* f) : _f(f) {}
   ~Lines() { free(_buf); }
   Lines(const Lines&) = delete;
   Lines& operator=(const Lines&) = delete;

   /* The next line without its '\n'; false at the end of the file. */
   bool next(std::string_view& line)
   {
      const ssize_t n = getline(&_buf, &_cap, _f);
      if ( n < 0 ) return false;
      ++_number;
      line = std::string_view(_buf, (size_t)n);
      if ( !line.empty() && line.back() == '\n' ) line.remove_suffix(1);
      return true;
   }
   long long number() const { return _number; }

private:
   FILE* _f;
   char* _buf {nullptr};
   size_t _cap {0};
   long long _number {0};
};

bool is_space(char c)
{
   return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f';
}

/* QString::splitRef(QRegExp("\\s+"), SkipEmptyParts) for ASCII white space. */
void split(std::string_view s, std::vector<std::string_view>& out)
{
   out.clear();
   size_t i = 0;
   while ( i < s.size() )
   {
      while ( i < s.size() && is_space(s[i]) ) ++i;
      size_t j = i;
      while ( j < s.size() && !is_space(s[j]) ) ++j;
      if ( j > i ) out.push_back(s.substr(i, j - i));
      i = j;
   }
}

bool equals_nocase(std::string_view a, const char* b)
{
   const size_t n = strlen(b);
   if ( a.size() != n ) return false;
   for ( size_t i = 0; i < n; ++i )
   {
      char c = a[i];
      if ( c >= 'A' && c <= 'Z' ) c = (char)(c - 'A' + 'a');
      if ( c != b[i] ) return false;
   }
   return true;
}

/* QString::toInt: an optional sign and decimal digits that fit an int; anything else is 0. */
int32_t to_int(std::string_view w)
{
   size_t i = 0;
   if ( !w.empty() && w[0] == '+' )
   {
      i = 1;
      if ( w.size() > 1 && w[1] == '-' ) return 0;
   }
   if ( i == w.size() ) return 0;
   int32_t v = 0;
   const char* e = w.data() + w.size();
   const auto r = std::from_chars(w.data() + i, e, v);
   return (r.ec == std::errc() && r.ptr == e) ? v : 0;
}

/* QString::toDouble in the C locale: an optional sign, decimal digits with an optional point
 * and exponent, or inf; nan without a sign. */
bool to_double(std::string_view w, double& out)
{
   size_t i = 0;
   bool neg = false;
   if ( !w.empty() && (w[0] == '+' || w[0] == '-') )
   {
      neg = w[0] == '-';
      i = 1;
   }
   const std::string_view body = w.substr(i);
   if ( equals_nocase(body, "inf") )
   {
      out = neg ? -HUGE_VAL : HUGE_VAL;
      return true;
   }
   if ( i == 0 && equals_nocase(body, "nan") )
   {
      out = std::nan("");
      return true;
   }
   if ( body.empty() || !((body[0] >= '0' && body[0] <= '9') || body[0] == '.') ) return false;
   double v = 0;
   const char* e = body.data() + body.size();
   const auto r = std::from_chars(body.data(), e, v, std::chars_format::general);
   if ( r.ec != std::errc() || r.ptr != e ) return false;
   out = neg ? -v : v;
   return true;
}

/* QString::toFloat: the double rounded to float, 0 when the field is not a number. */
float to_float(std::string_view w)
{
   double d = 0;
   return to_double(w, d) ? (float)d : 0.0f;
}

std::string str(std::string_view s)
{
   return std::string(s.substr(0, 200));
}

int write_names(const char* path, const std::vector<std::string>& names)
{
   if ( !path ) return KINC_SIM_OK;
   FILE* f = fopen(path, "wb");
   if ( !f ) return kinc_pm_fail(KINC_SIM_EINVAL, "cannot open %s for writing", path);
   bool ok = true;
   for ( const auto& n : names )
      ok = ok && fwrite(n.data(), 1, n.size(), f) == n.size() && fputc('\n', f) != EOF;
   ok = (fclose(f) == 0) && ok;
   return ok ? KINC_SIM_OK : kinc_pm_fail(KINC_SIM_EIO, "write to %s failed", path);
}

}  // namespace

int kinc_pm_read_names(const char* path, int64_t expected, const char* what, std::vector<std::string>& names)
{
   names.clear();
   if ( !path )
   {
      for ( int64_t i = 0; i < expected; ++i ) names.push_back(std::to_string(i));
      return KINC_SIM_OK;
   }
   FILE* f = fopen(path, "rb");
   if ( !f ) return kinc_pm_fail(KINC_SIM_EINVAL, "cannot open %s", path);
   Lines lines(f);
   std::string_view line;
   while ( lines.next(line) )
   {
      if ( !line.empty() && line.back() == '\r' ) line.remove_suffix(1);
      names.emplace_back(line);
   }
   const bool bad = ferror(f) != 0;
   fclose(f);
   if ( bad ) return kinc_pm_fail(KINC_SIM_EIO, "cannot read %s", path);
   if ( (int64_t)names.size() != expected )
      return kinc_pm_fail(KINC_SIM_EINVAL, "%s holds %lld names for %lld %s", path, (long long)names.size(),
                          (long long)expected, what);
   return KINC_SIM_OK;
}

/*
 * ImportCorrelationMatrix::process.  The reference's loop writes the pending pair again after
 * every line (its "save last pair" step sits inside the read loop), so a second line of any
 * file makes Matrix::write reject the repeated indent, and it skips lines of 2-10 fields while
 * rejecting empty ones, the reverse of what its comment states.  This reads what the loop is
 * written to read: consecutive lines of a pair are collected and the pair is written once, and
 * lines of 0 or 1 fields (empty lines, '#' markers) are skipped.  The checks, in the
 * reference's order: field count, mask length, pair index, cluster count.
 */
extern "C" int kinc_pm_import_text(const char* in_path, const char* ccm_path, const char* cmx_path, int32_t genes,
                                   int32_t max_clusters, int32_t samples, int32_t little_endian)
{
   if ( !in_path || !ccm_path || !cmx_path )
      return kinc_pm_fail(KINC_SIM_EINVAL, "Did not get valid input and/or output arguments.");
   if ( samples < 1 ) return kinc_pm_fail(KINC_SIM_EINVAL, "An integer argument given is less than the minimum.");
   FILE* in = fopen(in_path, "rb");
   if ( !in ) return kinc_pm_fail(KINC_SIM_EINVAL, "cannot open %s", in_path);
   kinc_pm *ccm = nullptr, *cmx = nullptr;
   int rc = kinc_pm_create(ccm_path, KINC_PM_CCM, genes, max_clusters, samples, little_endian, &ccm);
   if ( rc == KINC_SIM_OK ) rc = kinc_pm_create(cmx_path, KINC_PM_CMX, genes, max_clusters, 1, little_endian, &cmx);
   if ( rc != KINC_SIM_OK )
   {
      if ( ccm ) kinc_pm_close(ccm);
      fclose(in);
      return rc;
   }

   /* items waiting to be written, in pair order */
   std::vector<int32_t> cx, cy, mx, my;
   std::vector<int8_t> cc, mc, codes;
   std::vector<float> mr;
   /* the pair being read */
   int32_t px = 0, py = 0;
   int nclus = 0;
   int64_t last_pair = -1;
   std::vector<int8_t> pcodes;
   std::vector<float> pr;
   constexpr size_t BATCH = 1 << 16;

   auto flush = [&]() -> int {
      const auto vp = [](auto& v) { return (const void*)v.data(); };
      int r = kinc_pm_write_items(cmx, (int64_t)mx.size(), mx.data(), my.data(), mc.data(), vp(mr));
      if ( r == KINC_SIM_OK ) r = kinc_pm_write_items(ccm, (int64_t)cx.size(), cx.data(), cy.data(), cc.data(), vp(codes));
      mx.clear(), my.clear(), mc.clear(), mr.clear(), cx.clear(), cy.clear(), cc.clear(), codes.clear();
      return r;
   };
   auto close_pair = [&]() -> int {
      for ( int k = 0; k < nclus; ++k )
      {
         mx.push_back(px), my.push_back(py), mc.push_back((int8_t)k), mr.push_back(pr[(size_t)k]);
         if ( nclus > 1 ) cx.push_back(px), cy.push_back(py), cc.push_back((int8_t)k);
      }
      if ( nclus > 1 ) codes.insert(codes.end(), pcodes.begin(), pcodes.end());
      nclus = 0;
      pr.clear();
      pcodes.clear();
      return mx.size() >= BATCH ? flush() : KINC_SIM_OK;
   };

   Lines lines(in);
   std::string_view line;
   std::vector<std::string_view> w;
   while ( rc == KINC_SIM_OK && lines.next(line) )
   {
      split(line, w);
      if ( w.size() <= 1 ) continue;
      const long long ln = lines.number();
      if ( w.size() != 11 )
      {
         rc = kinc_pm_fail(KINC_SIM_EINVAL,
                           "Encountered line with incorrect amount of fields. Read %zu fields when there should "
                           "have been 11. (line %lld)", w.size(), ln);
         break;
      }
      const int32_t x = to_int(w[0]), y = to_int(w[1]);
      const float r = to_float(w[9]);
      const std::string_view mask = w[10];
      if ( (int64_t)mask.size() != samples )
      {
         rc = kinc_pm_fail(KINC_SIM_EINVAL, "Encountered sample mask with invalid length %zu. Sample size is %d. (line %lld)",
                           mask.size(), samples, ln);
         break;
      }
      if ( x < 1 || y < 0 || x <= y || x >= genes )
      {
         rc = kinc_pm_fail(KINC_SIM_EINVAL, "Cannot initialize pairwise index (%d, %d) of %d genes. (line %lld)", x, y,
                           genes, ln);
         break;
      }
      if ( nclus == 0 || x != px || y != py )
      {
         const int64_t pair = (int64_t)x * (x - 1) / 2 + y;
         if ( pair <= last_pair )
         {
            rc = kinc_pm_fail(KINC_SIM_EORDER, "Attempting to write indent %lld when last written is %lld. (line %lld)",
                              (long long)(pair * 64), (long long)(last_pair * 64 + (nclus > 0 ? nclus - 1 : 0)), ln);
            break;
         }
         if ( (rc = close_pair()) != KINC_SIM_OK ) break;
         px = x, py = y, last_pair = pair;
      }
      if ( nclus + 1 > max_clusters )
      {
         rc = kinc_pm_fail(KINC_SIM_EINVAL, "Cannot write pair with cluster size %d exceeding the max of %d. (line %lld)",
                           nclus + 1, max_clusters, ln);
         break;
      }
      pr.push_back(r);
      for ( char ch : mask ) pcodes.push_back((int8_t)(ch >= '0' && ch <= '9' ? ch - '0' : -1));
      ++nclus;
   }
   if ( rc == KINC_SIM_OK && ferror(in) ) rc = kinc_pm_fail(KINC_SIM_EIO, "cannot read %s", in_path);
   if ( rc == KINC_SIM_OK ) rc = close_pair();
   if ( rc == KINC_SIM_OK ) rc = flush();
   fclose(in);
   const int rc1 = kinc_pm_close(ccm), rc2 = kinc_pm_close(cmx);
   if ( rc == KINC_SIM_OK ) rc = rc1 ? rc1 : rc2;
   return rc;
}

/* ImportExpressionMatrix::process.  Each value is the double rounded to float, transformed by
 * the float overloads of log / log2 / log10 (the reference calls them on the float).  A line of
 * no fields is skipped (the reference's error message for it reads the first field of an empty
 * list). */
extern "C" int kinc_emx_import_text(const char* in_path, const char* nan_token, int32_t samples, int32_t transform,
                                    int32_t little_endian, const char* emx_path, const char* gene_names_path,
                                    const char* sample_names_path)
{
   if ( !in_path || !emx_path ) return kinc_pm_fail(KINC_SIM_EINVAL, "Did not get valid input and/or output arguments.");
   if ( samples < 0 ) return kinc_pm_fail(KINC_SIM_EINVAL, "An integer argument given is less than the minimum.");
   if ( transform < KINC_EMX_TRANSFORM_NONE || transform > KINC_EMX_TRANSFORM_LOG10 )
      return kinc_pm_fail(KINC_SIM_EINVAL, "transform %d is not one of 0..3", transform);
   const std::string_view token = nan_token ? nan_token : "";
   FILE* in = fopen(in_path, "rb");
   if ( !in ) return kinc_pm_fail(KINC_SIM_EINVAL, "cannot open %s", in_path);

   int64_t S = samples;
   std::vector<std::string> sample_names, gene_names;
   for ( int64_t i = 0; i < S; ++i ) sample_names.push_back(std::to_string(i));
   std::vector<float> gem;
   int rc = KINC_SIM_OK;
   Lines lines(in);
   std::string_view line;
   std::vector<std::string_view> w;
   while ( rc == KINC_SIM_OK && lines.next(line) )
   {
      split(line, w);
      if ( w.empty() ) continue;
      if ( S == 0 )
      {
         S = (int64_t)w.size();
         for ( auto s : w ) sample_names.emplace_back(s);
         continue;
      }
      if ( (int64_t)w.size() != S + 1 )
      {
         rc = kinc_pm_fail(KINC_SIM_EINVAL,
                           "Encountered gene expression line with incorrect amount of fields. Read in %lld fields "
                           "when it should have been %lld. Gene name is %s.",
                           (long long)w.size() - 1, (long long)S, str(w[0]).c_str());
         break;
      }
      for ( int64_t i = 1; i <= S; ++i )
      {
         if ( !token.empty() && w[(size_t)i] == token )
         {
            gem.push_back(std::nanf(""));
            continue;
         }
         double d = 0;
         if ( !to_double(w[(size_t)i], d) )
         {
            rc = kinc_pm_fail(KINC_SIM_EINVAL, "Failed to read expression value \"%s\" for gene %s.",
                              str(w[(size_t)i]).c_str(), str(w[0]).c_str());
            break;
         }
         const float v = (float)d;
         switch ( transform )
         {
         case KINC_EMX_TRANSFORM_NLOG: gem.push_back(std::log(v)); break;
         case KINC_EMX_TRANSFORM_LOG2: gem.push_back(std::log2(v)); break;
         case KINC_EMX_TRANSFORM_LOG10: gem.push_back(std::log10(v)); break;
         default: gem.push_back(v); break;
         }
      }
      gene_names.emplace_back(w[0]);
   }
   if ( rc == KINC_SIM_OK && ferror(in) ) rc = kinc_pm_fail(KINC_SIM_EIO, "cannot read %s", in_path);
   fclose(in);
   if ( rc != KINC_SIM_OK ) return rc;
   if ( gene_names.empty() || S < 1 ) return kinc_pm_fail(KINC_SIM_EINVAL, "%s holds no genes", in_path);
   if ( (int64_t)gene_names.size() > INT32_MAX || S > INT32_MAX )
      return kinc_pm_fail(KINC_SIM_EINVAL, "%s is larger than an expression matrix holds", in_path);
   if ( (rc = kinc_emx_write(emx_path, gem.data(), (int32_t)gene_names.size(), (int32_t)S, little_endian)) ) return rc;
   if ( (rc = write_names(gene_names_path, gene_names)) ) return rc;
   return write_names(sample_names_path, sample_names);
}

/* ExportExpressionMatrix::process.  The transform is undone with the reference's calls on the
 * float value: exp(float) (the float overload) and pow(2, float) / pow(10, float) (double,
 * rounded to float), and the float is printed at 12 significant digits. */
extern "C" int kinc_emx_export_text(const char* emx_path, int32_t little_endian, const char* gene_names_path,
                                    const char* sample_names_path, int32_t transform, const char* nan_token,
                                    const char* out_path)
{
   if ( !emx_path || !out_path ) return kinc_pm_fail(KINC_SIM_EINVAL, "Did not get valid input and/or output arguments.");
   if ( transform < KINC_EMX_TRANSFORM_NONE || transform > KINC_EMX_TRANSFORM_LOG10 )
      return kinc_pm_fail(KINC_SIM_EINVAL, "transform %d is not one of 0..3", transform);
   int32_t G = 0, S = 0;
   int rc = kinc_emx_read_header(emx_path, little_endian, &G, &S);
   if ( rc ) return rc;
   std::vector<float> gem((size_t)G * S);
   if ( (rc = kinc_emx_read(emx_path, little_endian, gem.data(), (int64_t)gem.size())) ) return rc;
   std::vector<std::string> gene_names, sample_names;
   if ( (rc = kinc_pm_read_names(gene_names_path, G, "genes", gene_names)) ) return rc;
   if ( (rc = kinc_pm_read_names(sample_names_path, S, "samples", sample_names)) ) return rc;
   const std::string token = nan_token ? nan_token : "";

   FILE* out = fopen(out_path, "wb");
   if ( !out ) return kinc_pm_fail(KINC_SIM_EINVAL, "cannot open %s for writing", out_path);
   std::vector<char> obuf(1 << 22);
   setvbuf(out, obuf.data(), _IOFBF, obuf.size());
   bool ok = true;
   for ( const auto& s : sample_names ) ok = ok && fputs(s.c_str(), out) != EOF && fputc('\t', out) != EOF;
   ok = ok && fputc('\n', out) != EOF;
   char num[64];
   for ( int32_t g = 0; ok && g < G; ++g )
   {
      ok = fputs(gene_names[(size_t)g].c_str(), out) != EOF;
      for ( int32_t s = 0; ok && s < S; ++s )
      {
         const float v = gem[(size_t)g * S + s];
         if ( std::isnan(v) )
         {
            ok = fputc('\t', out) != EOF && fputs(token.c_str(), out) != EOF;
            continue;
         }
         float w = v;
         switch ( transform )
         {
         case KINC_EMX_TRANSFORM_NLOG: w = std::exp(v); break;
         case KINC_EMX_TRANSFORM_LOG2: w = (float)std::pow(2.0, (double)v); break;
         case KINC_EMX_TRANSFORM_LOG10: w = (float)std::pow(10.0, (double)v); break;
         default: break;
         }
         /* to_chars with a precision prints as printf's %.12g does in the C locale */
         num[0] = '\t';
         const auto r = std::to_chars(num + 1, num + sizeof num, (double)w, std::chars_format::general, 12);
         ok = r.ec == std::errc() && fwrite(num, 1, (size_t)(r.ptr - num), out) == (size_t)(r.ptr - num);
      }
      ok = ok && fputc('\n', out) != EOF;
   }
   ok = (fclose(out) == 0) && ok;
   return ok ? KINC_SIM_OK : kinc_pm_fail(KINC_SIM_EIO, "write to %s failed", out_path);
}
