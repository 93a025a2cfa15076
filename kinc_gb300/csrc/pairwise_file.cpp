/*
 * pairwise_file.cpp -- CCM / CMX pairwise matrix files, EMX data, and the
 * ordered block runner (include/kinc_pairwise_matrix.h).
 *
 * Restates the on-disk behaviour of Pairwise::Matrix (src/core/pairwise_matrix.cpp:12-151,251-273),
 * CCMatrix::Pair::writeCluster/readCluster (src/core/ccmatrix.cpp:223-270),
 * CorrelationMatrix::Pair::writeCluster/readCluster (src/core/correlationmatrix.cpp:231-260) and
 * ExpressionMatrix's data section (src/core/expressionmatrix.cpp:21-37).
 */
#include "../../include/kinc_pairwise_matrix.h"
#include "sim_internal.h"

#include <cuda_runtime.h>
#include <unistd.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

namespace {

thread_local std::string t_err;

int pm_vfail(int code, const char* fmt, va_list ap)
{
   char buf[512];
   vsnprintf(buf, sizeof buf, fmt, ap);
   t_err = buf;
   return code;
}

__attribute__((format(printf, 2, 3))) int pm_fail(int code, const char* fmt, ...)
{
   va_list ap;
   va_start(ap, fmt);
   pm_vfail(code, fmt, ap);
   va_end(ap);
   return code;
}

constexpr int HEADER = 30;      /* Matrix::_headerSize */
constexpr int ITEM_HEADER = 9;  /* Matrix::_itemHeaderSize */
constexpr int MAX_CLUSTER_SIZE = 64;

/* byte-order-aware scalar I/O */
struct Endian
{
   bool little;

   template <class T>
   void put(std::vector<unsigned char>& out, T v) const
   {
      unsigned char b[sizeof(T)];
      memcpy(b, &v, sizeof(T));
      const bool host_little = true;   /* x86-64 and aarch64 builds are little-endian */
      if ( little != host_little )
         for ( size_t i = 0; i < sizeof(T) / 2; ++i ) std::swap(b[i], b[sizeof(T) - 1 - i]);
      out.insert(out.end(), b, b + sizeof(T));
   }

   template <class T>
   T get(const unsigned char* p) const
   {
      unsigned char b[sizeof(T)];
      memcpy(b, p, sizeof(T));
      if ( !little )
         for ( size_t i = 0; i < sizeof(T) / 2; ++i ) std::swap(b[i], b[sizeof(T) - 1 - i]);
      T v;
      memcpy(&v, b, sizeof(T));
      return v;
   }
};

}  // namespace

struct kinc_pm
{
   FILE* f = nullptr;
   bool writing = false;
   int type = 0;
   Endian e {};
   int32_t genes = 0, max_clusters = 0, subsize = 0, data_size = 0;
   int16_t offset = 0;
   int64_t pairs = 0, clusters = 0;
   int64_t last_indent = -1;
   int64_t last_pair = -1;
   std::unique_ptr<unsigned char[]> items;   /* item bytes of one write, not zero-filled */
   size_t items_cap = 0;
};

namespace {

int32_t data_size_of(int type, int32_t subsize)
{
   return type == KINC_PM_CCM ? (subsize + 1) / 2 : subsize * (int32_t)sizeof(float);
}

int16_t offset_of(int type)
{
   return type == KINC_PM_CCM ? 4 : 1;   /* CCMatrix / CorrelationMatrix DATA_OFFSET */
}

int write_header(kinc_pm* m)
{
   std::vector<unsigned char> h;
   m->e.put<int32_t>(h, m->genes);
   m->e.put<int32_t>(h, m->max_clusters);
   m->e.put<int32_t>(h, m->data_size);
   m->e.put<int64_t>(h, m->pairs);
   m->e.put<int64_t>(h, m->clusters);
   m->e.put<int16_t>(h, m->offset);
   if ( m->type == KINC_PM_CCM ) m->e.put<int32_t>(h, m->subsize);
   else m->e.put<int8_t>(h, (int8_t)m->subsize);
   if ( fseek(m->f, 0, SEEK_SET) != 0 || fwrite(h.data(), 1, h.size(), m->f) != h.size() )
      return pm_fail(KINC_SIM_EIO, "cannot write the pairwise matrix header");
   return KINC_SIM_OK;
}

}  // namespace

int kinc_pm_fail(int code, const char* fmt, ...)
{
   va_list ap;
   va_start(ap, fmt);
   pm_vfail(code, fmt, ap);
   va_end(ap);
   return code;
}

extern "C" const char* kinc_pm_last_error(void)
{
   return t_err.c_str();
}

extern "C" int kinc_pm_create(const char* path, int32_t type, int32_t genes, int32_t max_clusters, int32_t subsize,
                              int32_t little_endian, kinc_pm** out)
{
   if ( !path || !out ) return pm_fail(KINC_SIM_EINVAL, "path and out must not be NULL");
   *out = nullptr;
   if ( type != KINC_PM_CCM && type != KINC_PM_CMX ) return pm_fail(KINC_SIM_EINVAL, "type must be CCM or CMX");
   /* Matrix::initialize (src/core/pairwise_matrix.cpp:69-117) */
   if ( genes < 1 ) return pm_fail(KINC_SIM_EINVAL, "Gene names metadata is not an array or is empty.");
   if ( max_clusters < 1 || subsize < 1 )
      return pm_fail(KINC_SIM_EINVAL, "An integer argument given is less than the minimum.");
   if ( max_clusters > MAX_CLUSTER_SIZE )
      return pm_fail(KINC_SIM_EINVAL, "The max cluster size cannot be larger than MAX_CLUSTER_SIZE.");
   if ( type == KINC_PM_CMX && subsize > 127 ) return pm_fail(KINC_SIM_EINVAL, "correlationSize must fit in int8");
   kinc_pm* m = new kinc_pm();
   m->f = fopen(path, "w+b");
   if ( !m->f )
   {
      delete m;
      return pm_fail(KINC_SIM_EINVAL, "cannot open %s for writing", path);
   }
   m->writing = true;
   m->type = type;
   m->e.little = little_endian != 0;
   m->genes = genes;
   m->max_clusters = max_clusters;
   m->subsize = subsize;
   m->data_size = data_size_of(type, subsize);
   m->offset = offset_of(type);
   int rc = write_header(m);
   if ( rc )
   {
      fclose(m->f);
      delete m;
      return rc;
   }
   *out = m;
   return KINC_SIM_OK;
}

static int write_items(kinc_pm* m, int64_t n, const int32_t* x, const int32_t* y, const int8_t* c,
                       const void* payload, bool packed);

extern "C" int kinc_pm_write_items(kinc_pm* m, int64_t n, const int32_t* x, const int32_t* y, const int8_t* c,
                                   const void* payload)
{
   return write_items(m, n, x, y, c, payload, false);
}

extern "C" int kinc_pm_write_items_packed(kinc_pm* m, int64_t n, const int32_t* x, const int32_t* y,
                                          const int8_t* c, const void* payload)
{
   return write_items(m, n, x, y, c, payload, true);
}

static int write_items(kinc_pm* m, int64_t n, const int32_t* x, const int32_t* y, const int8_t* c,
                       const void* payload, bool packed)
{
   if ( !m || !m->writing ) return pm_fail(KINC_SIM_EINVAL, "Attempting to write data to uninitialized object.");
   if ( n < 0 || (n > 0 && (!x || !y || !c || !payload)) ) return pm_fail(KINC_SIM_EINVAL, "invalid item arrays");
   const size_t item = ITEM_HEADER + (size_t)m->data_size;
   /* validate the whole batch first so a rejected batch leaves the file as it was */
   {
      int64_t last = m->last_indent;
      for ( int64_t i = 0; i < n; ++i )
      {
         if ( x[i] < 1 || y[i] < 0 || x[i] <= y[i] || x[i] >= m->genes )
            return pm_fail(KINC_SIM_EINVAL, "Cannot initialize pairwise index (%d, %d).", x[i], y[i]);
         if ( c[i] < 0 || c[i] >= MAX_CLUSTER_SIZE || c[i] >= m->max_clusters )
            return pm_fail(KINC_SIM_EINVAL, "Cluster %d is outside limits.", c[i]);
         const int64_t pair = (int64_t)x[i] * (x[i] - 1) / 2 + y[i];
         const int64_t indent = pair * MAX_CLUSTER_SIZE + c[i];
         if ( indent <= last )
            return pm_fail(KINC_SIM_EORDER, "Attempting to write indent %lld when last written is %lld.",
                           (long long)(pair * MAX_CLUSTER_SIZE), (long long)last);
         last = indent;
      }
   }
   /* items are laid out straight into the buffer: 4-byte fields byte-swapped when the file's
    * order differs from the host's (x86-64 and aarch64, the hosts compiled for, are little-endian) */
   if ( (size_t)n * item > m->items_cap )
   {
      m->items.reset(new unsigned char[(size_t)n * item]);
      m->items_cap = (size_t)n * item;
   }
   const bool swap = !m->e.little;
   auto put32 = [swap](unsigned char* o, uint32_t v) {
      if ( swap ) v = __builtin_bswap32(v);
      memcpy(o, &v, 4);
   };
   unsigned char* o = m->items.get();
   for ( int64_t i = 0; i < n; ++i, o += item )
   {
      const int64_t pair = (int64_t)x[i] * (x[i] - 1) / 2 + y[i];
      const int64_t indent = pair * MAX_CLUSTER_SIZE + c[i];
      put32(o, (uint32_t)x[i]);
      put32(o + 4, (uint32_t)y[i]);
      o[8] = (unsigned char)c[i];
      unsigned char* d = o + ITEM_HEADER;
      if ( m->type == KINC_PM_CCM && packed )
      {
         memcpy(d, (const unsigned char*)payload + (size_t)i * m->data_size, (size_t)m->data_size);
      }
      else if ( m->type == KINC_PM_CCM )
      {
         const int8_t* codes = (const int8_t*)payload + (size_t)i * m->subsize;
         for ( int s = 0; s < m->subsize; s += 2 )
         {
            /* sample s in the low nibble, s + 1 in the high one (shifted as unsigned: a code
             * outside 0..15, such as a non-digit mask character's -1, keeps its low 4 bits) */
            unsigned v = (unsigned)(uint8_t)codes[s] & 0x0Fu;
            if ( s + 1 < m->subsize ) v |= ((unsigned)(uint8_t)codes[s + 1] << 4) & 0xF0u;
            d[s / 2] = (unsigned char)v;
         }
      }
      else
      {
         const float* r = (const float*)payload + (size_t)i * m->subsize;
         for ( int k = 0; k < m->subsize; ++k )
         {
            uint32_t bits;
            memcpy(&bits, &r[k], 4);
            put32(d + 4 * k, bits);
         }
      }
      if ( pair != m->last_pair )
      {
         ++m->pairs;
         m->last_pair = pair;
      }
      ++m->clusters;
      m->last_indent = indent;
   }
   const long pos = (long)(HEADER + m->offset) + (long)((m->clusters - n) * (int64_t)item);
   const size_t bytes = (size_t)n * item;
   if ( fseek(m->f, pos, SEEK_SET) != 0 || (bytes > 0 && fwrite(m->items.get(), 1, bytes, m->f) != bytes) )
      return pm_fail(KINC_SIM_EIO, "write failed");
   return KINC_SIM_OK;
}

extern "C" int kinc_pm_close(kinc_pm* m)
{
   if ( !m ) return KINC_SIM_EINVAL;
   int rc = KINC_SIM_OK;
   if ( m->writing ) rc = write_header(m);
   if ( m->f ) fclose(m->f);
   delete m;
   return rc;
}

extern "C" int kinc_pm_open(const char* path, int32_t type, int32_t little_endian, kinc_pm** out, int32_t* genes,
                            int32_t* max_clusters, int32_t* subsize, int64_t* pairs, int64_t* clusters)
{
   if ( !path || !out ) return pm_fail(KINC_SIM_EINVAL, "path and out must not be NULL");
   *out = nullptr;
   kinc_pm* m = new kinc_pm();
   m->f = fopen(path, "rb");
   if ( !m->f )
   {
      delete m;
      return pm_fail(KINC_SIM_EINVAL, "cannot open %s", path);
   }
   m->type = type;
   m->e.little = little_endian != 0;
   unsigned char h[HEADER + 4];
   const size_t want = HEADER + (type == KINC_PM_CCM ? 4 : 1);
   if ( fread(h, 1, want, m->f) != want )
   {
      fclose(m->f);
      delete m;
      return pm_fail(KINC_SIM_EINVAL, "%s: truncated header", path);
   }
   m->genes = m->e.get<int32_t>(h);
   m->max_clusters = m->e.get<int32_t>(h + 4);
   m->data_size = m->e.get<int32_t>(h + 8);
   m->pairs = m->e.get<int64_t>(h + 12);
   m->clusters = m->e.get<int64_t>(h + 20);
   m->offset = m->e.get<int16_t>(h + 28);
   m->subsize = type == KINC_PM_CCM ? m->e.get<int32_t>(h + 30) : (int32_t)(int8_t)h[30];
   if ( m->offset != offset_of(type) || m->data_size != data_size_of(type, m->subsize) )
   {
      fclose(m->f);
      delete m;
      return pm_fail(KINC_SIM_EINVAL, "%s: not a %s file with this byte order", path,
                     type == KINC_PM_CCM ? "CCM" : "CMX");
   }
   if ( genes ) *genes = m->genes;
   if ( max_clusters ) *max_clusters = m->max_clusters;
   if ( subsize ) *subsize = m->subsize;
   if ( pairs ) *pairs = m->pairs;
   if ( clusters ) *clusters = m->clusters;
   *out = m;
   return KINC_SIM_OK;
}

extern "C" int kinc_pm_read_items(kinc_pm* m, int64_t first, int64_t n, int32_t* x, int32_t* y, int8_t* c,
                                  void* payload)
{
   if ( !m || m->writing ) return pm_fail(KINC_SIM_EINVAL, "not opened for reading");
   if ( first < 0 || n < 0 || first + n > m->clusters ) return pm_fail(KINC_SIM_EINVAL, "item range out of bounds");
   const size_t item = ITEM_HEADER + (size_t)m->data_size;
   std::vector<unsigned char> b((size_t)n * item);
   const long pos = (long)(HEADER + m->offset) + (long)(first * (int64_t)item);
   if ( n > 0 && (fseek(m->f, pos, SEEK_SET) != 0 || fread(b.data(), 1, b.size(), m->f) != b.size()) )
      return pm_fail(KINC_SIM_EINVAL, "truncated items");
   for ( int64_t i = 0; i < n; ++i )
   {
      const unsigned char* p = b.data() + (size_t)i * item;
      if ( x ) x[i] = m->e.get<int32_t>(p);
      if ( y ) y[i] = m->e.get<int32_t>(p + 4);
      if ( c ) c[i] = (int8_t)p[8];
      if ( !payload ) continue;
      if ( m->type == KINC_PM_CCM )
      {
         int8_t* codes = (int8_t*)payload + (size_t)i * m->subsize;
         for ( int s = 0; s < m->subsize; ++s )
         {
            const unsigned char v = p[ITEM_HEADER + s / 2];
            codes[s] = (int8_t)((s % 2 == 0) ? (v & 0x0F) : ((v >> 4) & 0x0F));
         }
      }
      else
      {
         float* r = (float*)payload + (size_t)i * m->subsize;
         for ( int k = 0; k < m->subsize; ++k ) r[k] = m->e.get<float>(p + ITEM_HEADER + 4 * k);
      }
   }
   return KINC_SIM_OK;
}

extern "C" int kinc_emx_write(const char* path, const float* gem, int32_t genes, int32_t samples,
                              int32_t little_endian)
{
   if ( !path || !gem || genes < 1 || samples < 1 ) return pm_fail(KINC_SIM_EINVAL, "invalid EMX arguments");
   FILE* f = fopen(path, "wb");
   if ( !f ) return pm_fail(KINC_SIM_EINVAL, "cannot open %s for writing", path);
   Endian e { little_endian != 0 };
   std::vector<unsigned char> b;
   e.put<int32_t>(b, genes);
   e.put<int32_t>(b, samples);
   b.reserve(8 + (size_t)genes * samples * 4);
   for ( int64_t i = 0; i < (int64_t)genes * samples; ++i ) e.put<float>(b, gem[i]);
   const bool ok = fwrite(b.data(), 1, b.size(), f) == b.size();
   fclose(f);
   return ok ? KINC_SIM_OK : pm_fail(KINC_SIM_EIO, "write failed");
}

extern "C" int kinc_emx_read_header(const char* path, int32_t little_endian, int32_t* genes, int32_t* samples)
{
   FILE* f = path ? fopen(path, "rb") : nullptr;
   if ( !f ) return pm_fail(KINC_SIM_EINVAL, "cannot open EMX %s", path ? path : "(null)");
   unsigned char h[8];
   const bool ok = fread(h, 1, 8, f) == 8;
   fclose(f);
   if ( !ok ) return pm_fail(KINC_SIM_EINVAL, "%s: truncated EMX header", path);
   Endian e { little_endian != 0 };
   const int32_t g = e.get<int32_t>(h), s = e.get<int32_t>(h + 4);
   if ( g < 1 || s < 1 ) return pm_fail(KINC_SIM_EINVAL, "%s: corrupt EMX header (%d genes, %d samples)", path, g, s);
   if ( genes ) *genes = g;
   if ( samples ) *samples = s;
   return KINC_SIM_OK;
}

extern "C" int kinc_emx_read(const char* path, int32_t little_endian, float* gem, int64_t capacity)
{
   int32_t g = 0, s = 0;
   int rc = kinc_emx_read_header(path, little_endian, &g, &s);
   if ( rc ) return rc;
   if ( !gem || capacity < (int64_t)g * s ) return pm_fail(KINC_SIM_EINVAL, "EMX buffer too small");
   FILE* f = fopen(path, "rb");
   if ( !f ) return pm_fail(KINC_SIM_EINVAL, "cannot open EMX %s", path);
   std::vector<unsigned char> b((size_t)g * s * 4);
   const bool ok = fseek(f, 8, SEEK_SET) == 0 && fread(b.data(), 1, b.size(), f) == b.size();
   fclose(f);
   if ( !ok ) return pm_fail(KINC_SIM_EINVAL, "%s: truncated EMX data", path);
   Endian e { little_endian != 0 };
   for ( int64_t i = 0; i < (int64_t)g * s; ++i ) gem[i] = e.get<float>(b.data() + 4 * i);
   return KINC_SIM_OK;
}

/*
 * Resume point of an interrupted run (the runner writes work blocks in pair order and rewrites
 * the header counts only when it finishes, so an interrupted file holds a valid header, the
 * items of the finished blocks and possibly part of the next).  For each file that exists: the
 * items on disk are those that fit whole in its length; the work block of the last one may be
 * incomplete.  The resume block is the smallest such block over the files (first_block for a
 * file without items); both files are cut back to the items of the blocks before it and their
 * header counts are rewritten, so they are valid, finished files again.
 */
namespace {

int cut_back(const char* path, int type, bool little, int64_t* last_block_out, int64_t keep_before_pair,
             bool apply)
{
   FILE* f = fopen(path, apply ? "r+b" : "rb");
   if ( !f ) return pm_fail(KINC_SIM_EINVAL, "cannot open %s", path);
   Endian e { little };
   unsigned char h[HEADER + 4];
   const size_t hb = HEADER + (type == KINC_PM_CCM ? 4 : 1);
   if ( fread(h, 1, hb, f) != hb )
   {
      fclose(f);
      return pm_fail(KINC_SIM_EINVAL, "%s: truncated header", path);
   }
   const int32_t data_size = e.get<int32_t>(h + 8);
   const int16_t offset = e.get<int16_t>(h + 28);
   const int32_t subsize = type == KINC_PM_CCM ? e.get<int32_t>(h + 30) : (int32_t)(int8_t)h[30];
   if ( offset != offset_of(type) || data_size != data_size_of(type, subsize) )
   {
      fclose(f);
      return pm_fail(KINC_SIM_EINVAL, "%s: not a %s file with this byte order", path, type == KINC_PM_CCM ? "CCM" : "CMX");
   }
   const int64_t item = ITEM_HEADER + data_size;
   const int64_t base = HEADER + offset;
   fseek(f, 0, SEEK_END);
   const int64_t size = (int64_t)ftell(f);
   const int64_t n = size > base ? (size - base) / item : 0;
   auto pair_at = [&](int64_t i, int32_t* xo, int32_t* yo) -> int64_t {
      unsigned char b[8];
      if ( fseek(f, (long)(base + i * item), SEEK_SET) != 0 || fread(b, 1, 8, f) != 8 ) return -1;
      const int32_t x = e.get<int32_t>(b), y = e.get<int32_t>(b + 4);
      if ( xo ) *xo = x;
      if ( yo ) *yo = y;
      return (int64_t)x * (x - 1) / 2 + y;
   };
   if ( !apply )
   {
      int64_t last = -1;
      if ( n > 0 )
      {
         const int64_t p = pair_at(n - 1, nullptr, nullptr);
         if ( p < 0 )
         {
            fclose(f);
            return pm_fail(KINC_SIM_EIO, "cannot read %s", path);
         }
         last = p / KINC_SIM_WORK_BLOCK_SIZE;
      }
      *last_block_out = last;
      fclose(f);
      return KINC_SIM_OK;
   }
   /* keep the items whose pair is below keep_before_pair (items are in pair order) */
   int64_t lo = 0, hi = n;
   while ( lo < hi )
   {
      const int64_t mid = lo + (hi - lo) / 2;
      const int64_t p = pair_at(mid, nullptr, nullptr);
      if ( p < 0 )
      {
         fclose(f);
         return pm_fail(KINC_SIM_EIO, "cannot read %s", path);
      }
      if ( p < keep_before_pair ) lo = mid + 1;
      else hi = mid;
   }
   const int64_t keep = lo;
   /* the kept items' distinct pairs, read sequentially a chunk of items at a time */
   int64_t pairs = 0, prev = -1;
   {
      const int64_t per = std::max<int64_t>(1, (int64_t)(16u << 20) / item);
      std::vector<unsigned char> buf((size_t)(per * item));
      if ( fseek(f, (long)base, SEEK_SET) != 0 )
      {
         fclose(f);
         return pm_fail(KINC_SIM_EIO, "cannot read %s", path);
      }
      for ( int64_t i = 0; i < keep; i += per )
      {
         const int64_t len = std::min(per, keep - i);
         if ( fread(buf.data(), 1, (size_t)(len * item), f) != (size_t)(len * item) )
         {
            fclose(f);
            return pm_fail(KINC_SIM_EIO, "cannot read %s", path);
         }
         for ( int64_t j = 0; j < len; ++j )
         {
            const unsigned char* b = buf.data() + j * item;
            const int32_t x = e.get<int32_t>(b), y = e.get<int32_t>(b + 4);
            const int64_t p = (int64_t)x * (x - 1) / 2 + y;
            pairs += p != prev;
            prev = p;
         }
      }
   }
   std::vector<unsigned char> counts;
   e.put<int64_t>(counts, pairs);
   e.put<int64_t>(counts, keep);
   fflush(f);
   const bool ok = fseek(f, 12, SEEK_SET) == 0 && fwrite(counts.data(), 1, counts.size(), f) == counts.size()
                   && fflush(f) == 0 && ftruncate(fileno(f), (off_t)(base + keep * item)) == 0;
   fclose(f);
   return ok ? KINC_SIM_OK : pm_fail(KINC_SIM_EIO, "cannot cut %s back", path);
}

}  // namespace

extern "C" int kinc_pm_resume_point(const char* ccm_path, const char* cmx_path, int32_t little_endian,
                                    int64_t first_block, int64_t* resume_block)
{
   if ( !resume_block || first_block < 0 ) return pm_fail(KINC_SIM_EINVAL, "Did not get valid input and/or output arguments.");
   const char* paths[2] = { ccm_path, cmx_path };
   const int types[2] = { KINC_PM_CCM, KINC_PM_CMX };
   int64_t R = INT64_MAX;
   bool any = false;
   for ( int k = 0; k < 2; ++k )
   {
      if ( !paths[k] ) continue;
      if ( access(paths[k], F_OK) != 0 )
      {
         R = std::min(R, first_block);   /* nothing of this file was written */
         continue;
      }
      int64_t last = -1;
      const int rc = cut_back(paths[k], types[k], little_endian != 0, &last, 0, false);
      if ( rc ) return rc;
      any = true;
      R = std::min(R, last < 0 ? first_block : std::max(last, first_block));
   }
   if ( !any ) R = first_block;
   for ( int k = 0; k < 2; ++k )
   {
      if ( !paths[k] || access(paths[k], F_OK) != 0 ) continue;
      int64_t unused = 0;
      const int rc = cut_back(paths[k], types[k], little_endian != 0, &unused, R * KINC_SIM_WORK_BLOCK_SIZE, true);
      if ( rc ) return rc;
   }
   *resume_block = R;
   return KINC_SIM_OK;
}

/*
 * The files of a sharded run joined into one: each rank wrote the items of a contiguous range of
 * work blocks, so the joined file is the inputs' items back to back, in the order given.  The
 * inputs must agree on type, genes, maximum clusters and payload size, and their items must stay
 * in strictly increasing indent order across the joins (Matrix::write's rule); the header counts
 * are recomputed (a pair continued across a join counts once).
 */
namespace {

/* Append n items already encoded in the file's byte order (as another file of the same kind
 * holds them), with write_items' checks and bookkeeping. */
int append_raw_items(kinc_pm* m, const unsigned char* raw, int64_t n)
{
   const size_t item = ITEM_HEADER + (size_t)m->data_size;
   int64_t last = m->last_indent, last_pair = m->last_pair, pairs = m->pairs;
   for ( int64_t i = 0; i < n; ++i )
   {
      const unsigned char* o = raw + (size_t)i * item;
      const int32_t x = m->e.get<int32_t>(o), y = m->e.get<int32_t>(o + 4);
      const int c = (int8_t)o[8];
      if ( x < 1 || y < 0 || x <= y || x >= m->genes )
         return pm_fail(KINC_SIM_EINVAL, "Cannot initialize pairwise index (%d, %d).", x, y);
      if ( c < 0 || c >= MAX_CLUSTER_SIZE || c >= m->max_clusters )
         return pm_fail(KINC_SIM_EINVAL, "Cluster %d is outside limits.", c);
      const int64_t pair = (int64_t)x * (x - 1) / 2 + y;
      const int64_t indent = pair * MAX_CLUSTER_SIZE + c;
      if ( indent <= last )
         return pm_fail(KINC_SIM_EORDER, "Attempting to write indent %lld when last written is %lld.",
                        (long long)(pair * MAX_CLUSTER_SIZE), (long long)last);
      last = indent;
      if ( pair != last_pair )
      {
         ++pairs;
         last_pair = pair;
      }
   }
   const long pos = (long)(HEADER + m->offset) + (long)(m->clusters * (int64_t)item);
   const size_t bytes = (size_t)n * item;
   if ( fseek(m->f, pos, SEEK_SET) != 0 || (bytes > 0 && fwrite(raw, 1, bytes, m->f) != bytes) )
      return pm_fail(KINC_SIM_EIO, "write failed");
   m->last_indent = last;
   m->last_pair = last_pair;
   m->pairs = pairs;
   m->clusters += n;
   return KINC_SIM_OK;
}

}  // namespace

extern "C" int kinc_pm_concat(const char* out_path, const char* const* in_paths, int32_t n, int32_t little_endian)
{
   if ( !out_path || !in_paths || n < 1 ) return pm_fail(KINC_SIM_EINVAL, "Did not get valid input and/or output arguments.");
   for ( int32_t i = 0; i < n; ++i )
   {
      if ( !in_paths[i] ) return pm_fail(KINC_SIM_EINVAL, "input %d is NULL", i);
      char a[4096], b[4096];
      if ( realpath(in_paths[i], a) && realpath(out_path, b) && strcmp(a, b) == 0 )
         return pm_fail(KINC_SIM_EINVAL, "the output %s is also input %d", out_path, i);
   }
   int type = 0;
   int32_t G = 0, K = 0, sub = 0;
   for ( int t : { KINC_PM_CCM, KINC_PM_CMX } )
   {
      kinc_pm* m = nullptr;
      if ( kinc_pm_open(in_paths[0], t, little_endian, &m, &G, &K, &sub, nullptr, nullptr) == KINC_SIM_OK )
      {
         kinc_pm_close(m);
         type = t;
         break;
      }
   }
   if ( !type ) return pm_fail(KINC_SIM_EINVAL, "%s is neither a CCM nor a CMX file in this byte order", in_paths[0]);
   kinc_pm* out = nullptr;
   int rc = kinc_pm_create(out_path, type, G, K, sub, little_endian, &out);
   if ( rc ) return rc;
   /* items are copied as they are encoded (the files share one byte order), a chunk at a time */
   const int64_t item = ITEM_HEADER + (int64_t)out->data_size;
   const int64_t chunk = std::max<int64_t>(1, (int64_t)(32u << 20) / item);
   std::vector<unsigned char> buf((size_t)(chunk * item));
   for ( int32_t i = 0; i < n && rc == KINC_SIM_OK; ++i )
   {
      kinc_pm* m = nullptr;
      int32_t g = 0, k = 0, s2 = 0;
      int64_t items = 0;
      if ( (rc = kinc_pm_open(in_paths[i], type, little_endian, &m, &g, &k, &s2, nullptr, &items)) ) break;
      if ( g != G || k != K || s2 != sub )
      {
         rc = pm_fail(KINC_SIM_EINVAL, "%s (%d genes, %d clusters, %d per item) does not match %s (%d, %d, %d)",
                      in_paths[i], g, k, s2, in_paths[0], G, K, sub);
      }
      if ( rc == KINC_SIM_OK && fseek(m->f, (long)(HEADER + m->offset), SEEK_SET) != 0 )
         rc = pm_fail(KINC_SIM_EIO, "cannot read %s", in_paths[i]);
      for ( int64_t first = 0; rc == KINC_SIM_OK && first < items; first += chunk )
      {
         const int64_t len = std::min(chunk, items - first);
         if ( fread(buf.data(), 1, (size_t)(len * item), m->f) != (size_t)(len * item) )
            rc = pm_fail(KINC_SIM_EINVAL, "%s: truncated items", in_paths[i]);
         else
            rc = append_raw_items(out, buf.data(), len);
      }
      kinc_pm_close(m);
   }
   const int rc2 = kinc_pm_close(out);
   if ( rc || rc2 ) remove(out_path);   /* no half-joined file is left behind */
   return rc ? rc : rc2;
}

/*
 * ExportCorrelationMatrix::process (src/core/exportcorrelationmatrix.cpp:17-117): one text line
 * per CMX cluster, "x y k clusterSize samples missing postOutliers preOutliers threshold r mask"
 * separated by tabs.  The counts and the sample mask come from the CCM cluster only when the
 * CMX pair has more than one cluster (else zeros and a mask of '0's); r is the cluster's first
 * correlation, printed as the reference's text stream prints a float at precision 6 (%.6g of its
 * double value).  CMX and CCM are both in pair order, so the CCM pair is found by walking a
 * second cursor forward.
 */
extern "C" int kinc_pm_export_text(const char* ccm_path, const char* cmx_path, int32_t little_endian,
                                   const char* out_path)
{
   if ( !ccm_path || !cmx_path || !out_path )
      return pm_fail(KINC_SIM_EINVAL, "Did not get valid input and/or output arguments.");
   kinc_pm *cmx = nullptr, *ccm = nullptr;
   int32_t g1 = 0, k1 = 0, nc = 0, g2 = 0, k2 = 0, S = 0;
   int64_t p1 = 0, n_cmx = 0, p2 = 0, n_ccm = 0;
   int rc = kinc_pm_open(cmx_path, KINC_PM_CMX, little_endian, &cmx, &g1, &k1, &nc, &p1, &n_cmx);
   if ( rc ) return rc;
   if ( (rc = kinc_pm_open(ccm_path, KINC_PM_CCM, little_endian, &ccm, &g2, &k2, &S, &p2, &n_ccm)) )
   {
      kinc_pm_close(cmx);
      return rc;
   }
   FILE* out = fopen(out_path, "wb");
   if ( !out )
   {
      kinc_pm_close(cmx);
      kinc_pm_close(ccm);
      return pm_fail(KINC_SIM_EINVAL, "cannot open %s for writing", out_path);
   }
   std::vector<char> obuf(1 << 22);
   setvbuf(out, obuf.data(), _IOFBF, obuf.size());

   constexpr int64_t CHUNK = 1 << 16;
   /* CMX items, read a chunk at a time */
   std::vector<int32_t> ax(CHUNK), ay(CHUNK);
   std::vector<int8_t> ac(CHUNK);
   std::vector<float> ar((size_t)CHUNK * nc);
   int64_t a_base = 0, a_len = 0;
   /* CCM items: a window that always starts at the cursor */
   std::vector<int32_t> bx(CHUNK), by(CHUNK);
   std::vector<int8_t> bc(CHUNK);
   std::vector<int8_t> bcodes((size_t)CHUNK * S);
   int64_t b_base = 0, b_len = 0, b_cur = 0;
   std::string mask((size_t)S, '0'), lbuf;
   std::vector<int8_t> codes;   /* the CCM clusters of the current pair, [cluster][S] */
   std::vector<float> r;        /* the current pair's first correlations */
   char line[256];

   auto fill_ccm = [&](int64_t first) -> int {
      b_base = first;
      b_len = std::min<int64_t>(CHUNK, n_ccm - first);
      if ( b_len <= 0 ) return KINC_SIM_OK;
      return kinc_pm_read_items(ccm, first, b_len, bx.data(), by.data(), bc.data(), bcodes.data());
   };
   auto pair_of = [](int32_t x, int32_t y) { return (int64_t)x * (x - 1) / 2 + y; };

   int64_t i = 0;
   while ( rc == KINC_SIM_OK && i < n_cmx )
   {
      /* the CMX pair starting at item i: its clusters are items [i, j) */
      auto at = [&](int64_t q) -> int64_t {
         if ( q < a_base || q >= a_base + a_len )
         {
            a_base = q;
            a_len = std::min<int64_t>(CHUNK, n_cmx - q);
            if ( kinc_pm_read_items(cmx, q, a_len, ax.data(), ay.data(), ac.data(), ar.data()) ) return -1;
         }
         return q - a_base;
      };
      int64_t o = at(i);
      if ( o < 0 ) { rc = KINC_SIM_EINVAL; break; }
      const int32_t x = ax[o], y = ay[o];
      r.clear();
      int64_t j = i;
      while ( j < n_cmx )
      {
         const int64_t q = at(j);
         if ( q < 0 ) { rc = KINC_SIM_EINVAL; break; }
         if ( ax[q] != x || ay[q] != y ) break;
         r.push_back(ar[(size_t)q * nc]);
         ++j;
      }
      if ( rc ) break;
      const int clusters = (int)(j - i);
      codes.clear();
      if ( clusters > 1 )
      {
         /* advance the CCM cursor to this pair and collect its clusters */
         const int64_t want = pair_of(x, y);
         for ( ;; )
         {
            if ( b_cur >= n_ccm ) break;
            if ( b_cur < b_base || b_cur >= b_base + b_len )
               if ( (rc = fill_ccm(b_cur)) ) break;
            const int64_t q = b_cur - b_base;
            const int64_t have = pair_of(bx[q], by[q]);
            if ( have < want ) { ++b_cur; continue; }
            if ( have > want ) break;
            codes.insert(codes.end(), bcodes.begin() + q * S, bcodes.begin() + (q + 1) * S);
            ++b_cur;
         }
         if ( rc ) break;
         if ( (int)(codes.size() / (size_t)std::max(S, 1)) < clusters )
         {
            rc = pm_fail(KINC_SIM_EINVAL, "CCM holds %zu clusters for pair (%d, %d), CMX %d",
                         codes.size() / (size_t)std::max(S, 1), x, y, clusters);
            break;
         }
      }
      for ( int k = 0; k < clusters; ++k )
      {
         /* per-code counts from a 16-bin histogram of the cluster's nibbles */
         int hist[16] = { 0 };
         if ( clusters > 1 )
         {
            const int8_t* c = codes.data() + (size_t)k * S;
            for ( int s2 = 0; s2 < S; ++s2 )
            {
               ++hist[c[s2] & 15];
               mask[(size_t)s2] = (char)('0' + c[s2]);
            }
         }
         else
         {
            std::fill(mask.begin(), mask.end(), '0');
         }
         const int n = snprintf(line, sizeof line, "%d\t%d\t%d\t%d\t%d\t%d\t%d\t%d\t%d\t%.6g\t", x, y, k, clusters, hist[1],
                                hist[9], hist[8], hist[7], hist[6], (double)r[(size_t)k]);
         /* the whole line in one write */
         lbuf.assign(line, (size_t)n);
         lbuf.append(mask);
         lbuf.push_back('\n');
         if ( fwrite(lbuf.data(), 1, lbuf.size(), out) != lbuf.size() )
         {
            rc = pm_fail(KINC_SIM_EIO, "write to %s failed", out_path);
            break;
         }
      }
      i = j;
   }
   if ( fclose(out) != 0 && rc == KINC_SIM_OK ) rc = pm_fail(KINC_SIM_EIO, "write to %s failed", out_path);
   kinc_pm_close(cmx);
   kinc_pm_close(ccm);
   return rc;
}

/*
 * Extract::process (src/core/extract.cpp:24-274): the network of the clusters whose first
 * correlation r has mincorr <= |r| <= maxcorr, as a tab-separated edge list (header line, then
 * "source target r co cluster clusters samples missing postOutliers preOutliers threshold mask")
 * and as GraphML (every gene a node, every kept cluster an undirected edge with its sample
 * mask).  Multi-cluster pairs take counts and mask from the CCM; single-cluster pairs take the
 * mask from the expression matrix ('9' where either gene is NaN, else '1') and zero counts, as
 * the reference does.  Gene names are read from names_path (one per line) when given, else the
 * gene indices are the names.  Both outputs come from one walk over the CMX.
 */
extern "C" int kinc_pm_extract(const char* emx_path, const char* ccm_path, const char* cmx_path,
                               const char* names_path, int32_t little_endian, float min_corr, float max_corr,
                               const char* tsv_path, const char* graphml_path)
{
   if ( !emx_path || !ccm_path || !cmx_path || (!tsv_path && !graphml_path) )
      return pm_fail(KINC_SIM_EINVAL, "Did not get valid input and/or output arguments.");
   int32_t G = 0, S = 0;
   int rc = kinc_emx_read_header(emx_path, little_endian, &G, &S);
   if ( rc ) return rc;
   std::vector<float> gem((size_t)G * S);
   if ( (rc = kinc_emx_read(emx_path, little_endian, gem.data(), (int64_t)gem.size())) ) return rc;
   std::vector<std::string> names;
   if ( (rc = kinc_pm_read_names(names_path, G, "genes", names)) ) return rc;

   kinc_pm *cmx = nullptr, *ccm = nullptr;
   int32_t g1 = 0, k1 = 0, nc = 0, g2 = 0, k2 = 0, S2 = 0;
   int64_t p1 = 0, n_cmx = 0, p2 = 0, n_ccm = 0;
   if ( (rc = kinc_pm_open(cmx_path, KINC_PM_CMX, little_endian, &cmx, &g1, &k1, &nc, &p1, &n_cmx)) ) return rc;
   if ( (rc = kinc_pm_open(ccm_path, KINC_PM_CCM, little_endian, &ccm, &g2, &k2, &S2, &p2, &n_ccm)) )
   {
      kinc_pm_close(cmx);
      return rc;
   }
   if ( g1 != G || g2 != G || S2 != S )
   {
      kinc_pm_close(cmx);
      kinc_pm_close(ccm);
      return pm_fail(KINC_SIM_EINVAL, "EMX %d x %d, CMX %d genes, CCM %d genes x %d samples do not match", G, S, g1, g2,
                     S2);
   }
   FILE* tsv = tsv_path ? fopen(tsv_path, "wb") : nullptr;
   FILE* gml = graphml_path ? fopen(graphml_path, "wb") : nullptr;
   if ( (tsv_path && !tsv) || (graphml_path && !gml) )
   {
      if ( tsv ) fclose(tsv);
      if ( gml ) fclose(gml);
      kinc_pm_close(cmx);
      kinc_pm_close(ccm);
      return pm_fail(KINC_SIM_EINVAL, "cannot open the output files");
   }
   std::vector<char> tb(1 << 22), gb(1 << 22);
   if ( tsv ) setvbuf(tsv, tb.data(), _IOFBF, tb.size());
   if ( gml ) setvbuf(gml, gb.data(), _IOFBF, gb.size());
   bool io_ok = true;
   auto put = [&](FILE* f, const std::string& str) {
      if ( f && fwrite(str.data(), 1, str.size(), f) != str.size() ) io_ok = false;
   };
   put(tsv, "Source\tTarget\tsc\tInteraction\tCluster\tNum_Clusters\tCluster_Samples\tMissing_Samples\t"
            "Cluster_Outliers\tPair_Outliers\tToo_Low\tSamples\n");
   put(gml, "<?xml version=\"1.0\" encoding=\"UTF-8\"?>\n"
            "<graphml xmlns=\"http://graphml.graphdrawing.org/xmlns\"\n"
            "    xmlns:xsi=\"http://www.w3.org/2001/XMLSchema-instance\"\n"
            "    xsi:schemaLocation=\"http://graphml.graphdrawing.org/xmlns/1.0/graphml.xsd\">\n"
            "  <graph id=\"G\" edgedefault=\"undirected\">\n");
   for ( int32_t g = 0; g < G && gml; ++g ) put(gml, "    <node id=\"" + names[(size_t)g] + "\"/>\n");

   constexpr int64_t CHUNK = 1 << 16;
   std::vector<int32_t> ax(CHUNK), ay(CHUNK), bx(CHUNK), by(CHUNK);
   std::vector<int8_t> ac(CHUNK), bc(CHUNK), bcodes((size_t)CHUNK * S);
   std::vector<float> ar((size_t)CHUNK * nc);
   int64_t a_base = 0, a_len = 0, b_base = 0, b_len = 0, b_cur = 0;
   std::vector<int8_t> codes;
   std::vector<float> r;        /* the current pair's first correlations */
   std::string mask((size_t)S, '0');
   char num[64];
   auto pair_of = [](int32_t x, int32_t y) { return (int64_t)x * (x - 1) / 2 + y; };
   auto at = [&](int64_t q) -> int64_t {
      if ( q < a_base || q >= a_base + a_len )
      {
         a_base = q;
         a_len = std::min<int64_t>(CHUNK, n_cmx - q);
         if ( kinc_pm_read_items(cmx, q, a_len, ax.data(), ay.data(), ac.data(), ar.data()) ) return -1;
      }
      return q - a_base;
   };

   int64_t i = 0;
   while ( rc == KINC_SIM_OK && io_ok && i < n_cmx )
   {
      int64_t o = at(i);
      if ( o < 0 ) { rc = KINC_SIM_EINVAL; break; }
      const int32_t x = ax[o], y = ay[o];
      if ( x >= G || y >= G ) { rc = pm_fail(KINC_SIM_EINVAL, "pair (%d, %d) outside %d genes", x, y, G); break; }
      r.clear();
      int64_t j = i;
      while ( j < n_cmx )
      {
         const int64_t q = at(j);
         if ( q < 0 ) { rc = KINC_SIM_EINVAL; break; }
         if ( ax[q] != x || ay[q] != y ) break;
         r.push_back(ar[(size_t)q * nc]);
         ++j;
      }
      if ( rc ) break;
      const int clusters = (int)(j - i);
      codes.clear();
      if ( clusters > 1 )
      {
         const int64_t want = pair_of(x, y);
         for ( ;; )
         {
            if ( b_cur >= n_ccm ) break;
            if ( b_cur < b_base || b_cur >= b_base + b_len )
            {
               b_base = b_cur;
               b_len = std::min<int64_t>(CHUNK, n_ccm - b_cur);
               if ( (rc = kinc_pm_read_items(ccm, b_base, b_len, bx.data(), by.data(), bc.data(), bcodes.data())) ) break;
            }
            const int64_t q = b_cur - b_base;
            const int64_t have = pair_of(bx[q], by[q]);
            if ( have < want ) { ++b_cur; continue; }
            if ( have > want ) break;
            codes.insert(codes.end(), bcodes.begin() + q * S, bcodes.begin() + (q + 1) * S);
            ++b_cur;
         }
         if ( rc ) break;
         if ( (int)(codes.size() / (size_t)std::max(S, 1)) < clusters )
         {
            rc = pm_fail(KINC_SIM_EINVAL, "CCM holds %zu clusters for pair (%d, %d), CMX %d",
                         codes.size() / (size_t)std::max(S, 1), x, y, clusters);
            break;
         }
      }
      for ( int k = 0; k < clusters; ++k )
      {
         const float corr = r[(size_t)k];
         if ( fabsf(corr) < min_corr || max_corr < fabsf(corr) ) continue;
         /* per-code counts from a 16-bin histogram of the cluster's nibbles */
         int hist[16] = { 0 };
         if ( clusters > 1 )
         {
            const int8_t* c = codes.data() + (size_t)k * S;
            for ( int s2 = 0; s2 < S; ++s2 )
            {
               ++hist[c[s2] & 15];
               mask[(size_t)s2] = (char)('0' + c[s2]);
            }
         }
         else
         {
            const float* gx = gem.data() + (size_t)x * S;
            const float* gy = gem.data() + (size_t)y * S;
            for ( int s2 = 0; s2 < S; ++s2 ) mask[(size_t)s2] = (std::isnan(gx[s2]) || std::isnan(gy[s2])) ? '9' : '1';
         }
         const std::string& src = names[(size_t)x];
         const std::string& dst = names[(size_t)y];
         if ( tsv )
         {
            snprintf(num, sizeof num, "%.6g", (double)corr);
            std::string line;
            line.reserve(96 + src.size() + dst.size() + (size_t)S);
            line += src; line += '\t'; line += dst; line += '\t'; line += num; line += "\tco\t";
            line += std::to_string(k); line += '\t'; line += std::to_string(clusters); line += '\t';
            line += std::to_string(hist[1]); line += '\t'; line += std::to_string(hist[9]); line += '\t';
            line += std::to_string(hist[8]); line += '\t'; line += std::to_string(hist[7]); line += '\t';
            line += std::to_string(hist[6]); line += '\t'; line += mask; line += '\n';
            put(tsv, line);
         }
         if ( gml ) put(gml, "    <edge source=\"" + src + "\" target=\"" + dst + "\" samples=\"" + mask + "\"/>\n");
      }
      i = j;
   }
   put(gml, "  </graph>\n</graphml>\n");
   if ( tsv && fclose(tsv) != 0 ) io_ok = false;
   if ( gml && fclose(gml) != 0 ) io_ok = false;
   kinc_pm_close(cmx);
   kinc_pm_close(ccm);
   if ( rc == KINC_SIM_OK && !io_ok ) rc = pm_fail(KINC_SIM_EIO, "writing the network files failed");
   return rc;
}

namespace {

/* One of the runner's two result slots: a device block's results, its compacted
 * items on the device and their pinned host copies. */
struct RunSlot
{
   int8_t* dK = nullptr;
   int8_t* dL = nullptr;
   float* dC = nullptr;
   int32_t *dCx = nullptr, *dCy = nullptr, *dMx = nullptr, *dMy = nullptr;
   int8_t *dCc = nullptr, *dMc = nullptr;
   float* dCr = nullptr;
   uint8_t* dMp = nullptr;
   int32_t *hCx = nullptr, *hCy = nullptr, *hMx = nullptr, *hMy = nullptr;
   int8_t *hCc = nullptr, *hMc = nullptr;
   float* hCr = nullptr;
   uint8_t* hMp = nullptr;
   uint64_t* dCount = nullptr;
   uint64_t* hCount = nullptr;   /* [0] CMX items, [1] CCM items, [2] kernel status */
   cudaEvent_t counted = nullptr;
   int64_t cap = 0, start = 0, size = 0;

   void free_items()
   {
      cudaFree(dCx); cudaFree(dCy); cudaFree(dCc); cudaFree(dCr);
      cudaFree(dMx); cudaFree(dMy); cudaFree(dMc); cudaFree(dMp);
      cudaFreeHost(hCx); cudaFreeHost(hCy); cudaFreeHost(hCc); cudaFreeHost(hCr);
      cudaFreeHost(hMx); cudaFreeHost(hMy); cudaFreeHost(hMc); cudaFreeHost(hMp);
      dCx = dCy = dMx = dMy = hCx = hCy = hMx = hMy = nullptr;
      dCc = dMc = hCc = hMc = nullptr;
      dCr = hCr = nullptr;
      dMp = hMp = nullptr;
      cap = 0;
   }

   bool alloc_items(int64_t n, int ncorr, bool ccm, int nbytes)
   {
      free_items();
      bool ok = cudaMalloc(&dCx, n * 4) == cudaSuccess && cudaMalloc(&dCy, n * 4) == cudaSuccess
                && cudaMalloc(&dCc, n) == cudaSuccess && cudaMalloc(&dCr, n * 4 * ncorr) == cudaSuccess
                && cudaMallocHost(&hCx, n * 4) == cudaSuccess && cudaMallocHost(&hCy, n * 4) == cudaSuccess
                && cudaMallocHost(&hCc, n) == cudaSuccess && cudaMallocHost(&hCr, n * 4 * ncorr) == cudaSuccess;
      if ( ok && ccm )
         ok = cudaMalloc(&dMx, n * 4) == cudaSuccess && cudaMalloc(&dMy, n * 4) == cudaSuccess
              && cudaMalloc(&dMc, n) == cudaSuccess && cudaMalloc(&dMp, (size_t)n * nbytes) == cudaSuccess
              && cudaMallocHost(&hMx, n * 4) == cudaSuccess && cudaMallocHost(&hMy, n * 4) == cudaSuccess
              && cudaMallocHost(&hMc, n) == cudaSuccess && cudaMallocHost(&hMp, (size_t)n * nbytes) == cudaSuccess;
      cap = ok ? n : 0;
      return ok;
   }

   void release()
   {
      free_items();
      cudaFree(dK); cudaFree(dL); cudaFree(dC); cudaFree(dCount); cudaFreeHost(hCount);
      if ( counted ) cudaEventDestroy(counted);
      dK = dL = nullptr;
      dC = nullptr;
      dCount = hCount = nullptr;
      counted = nullptr;
   }
};

}  // namespace

extern "C" int kinc_sim_run_to_files(kinc_sim_ctx* ctx, const char* ccm_path, const char* cmx_path,
                                     int32_t little_endian, int64_t first_block, int64_t nblocks)
{
   return kinc_sim_run_to_files_ex(ctx, ccm_path, cmx_path, little_endian, first_block, nblocks, 0);
}

extern "C" int kinc_sim_run_to_files_ex(kinc_sim_ctx* ctx, const char* ccm_path, const char* cmx_path,
                                        int32_t little_endian, int64_t first_block, int64_t nblocks,
                                        int64_t device_block)
{
   kinc_sim_params p;
   int32_t G = 0, S = 0;
   if ( !ctx || kinc_sim_get_params(ctx, &p, &G, &S) != KINC_SIM_OK ) return pm_fail(KINC_SIM_EINVAL, "no context");
   const int64_t total = kinc_sim_total_pairs(ctx);
   const int64_t nb = kinc_sim_num_work_blocks(ctx);
   if ( first_block < 0 || first_block > nb ) return pm_fail(KINC_SIM_EINVAL, "first_block out of range");
   const int64_t max_dev = kinc_sim_max_device_block(ctx);
   if ( device_block < 0 || device_block > std::max<int64_t>(max_dev, KINC_SIM_WORK_BLOCK_SIZE) )
      return pm_fail(KINC_SIM_EINVAL, "device_block %lld outside [0, %lld]", (long long)device_block,
                     (long long)max_dev);
   const int64_t last_block = nblocks < 0 ? nb : std::min<int64_t>(nb, first_block + nblocks);
   const int64_t pair0 = first_block * KINC_SIM_WORK_BLOCK_SIZE;
   const int64_t pair1 = std::min<int64_t>(total, last_block * KINC_SIM_WORK_BLOCK_SIZE);
   const int maxK = p.max_clusters;
   const int ncorr = p.corr_method == 2 ? 2 : 1;
   const bool want_ccm = ccm_path != nullptr && p.clus_method != 0;
   kinc_pm* ccm = nullptr;
   kinc_pm* cmx = nullptr;
   int rc = KINC_SIM_OK;
   if ( ccm_path && (rc = kinc_pm_create(ccm_path, KINC_PM_CCM, G, maxK, S, little_endian, &ccm)) ) return rc;
   if ( cmx_path && (rc = kinc_pm_create(cmx_path, KINC_PM_CMX, G, maxK, ncorr, little_endian, &cmx)) )
   {
      if ( ccm ) kinc_pm_close(ccm);
      return rc;
   }
   /*
    * Device blocks of whole work blocks, in two slots: while the GPU computes
    * block b into one slot, block b-1's kept items (filtered and compacted on
    * the GPU, Similarity::process, src/core/similarity.cpp:66-127) come back
    * from the other slot on a copy stream into pinned buffers and are appended
    * to the files in pair order.
    */
   const int64_t B = std::max<int64_t>(KINC_SIM_WORK_BLOCK_SIZE,
                                       (device_block > 0 ? device_block : max_dev) / KINC_SIM_WORK_BLOCK_SIZE
                                          * KINC_SIM_WORK_BLOCK_SIZE);
   const int64_t Bn = std::min<int64_t>(B, std::max<int64_t>(pair1 - pair0, 1));
   const int nbytes = (S + 1) / 2;
   cudaStream_t st = nullptr, cs = nullptr;
   RunSlot slot[2];
   bool ok = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess
             && cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) == cudaSuccess;
   for ( int i = 0; i < 2 && ok; ++i )
   {
      RunSlot& s = slot[i];
      ok = cudaMalloc(&s.dK, Bn) == cudaSuccess
           && cudaMalloc(&s.dC, (size_t)Bn * maxK * ncorr * sizeof(float)) == cudaSuccess
           && (!want_ccm || cudaMalloc(&s.dL, (size_t)Bn * S) == cudaSuccess)
           && cudaMalloc(&s.dCount, 3 * sizeof(uint64_t)) == cudaSuccess
           && cudaMallocHost(&s.hCount, 3 * sizeof(uint64_t)) == cudaSuccess
           && cudaEventCreateWithFlags(&s.counted, cudaEventDisableTiming) == cudaSuccess
           /* item buffers start at 2^21 (or every cluster of the block) and grow on demand */
           && s.alloc_items(std::min<int64_t>(Bn * maxK, (int64_t)1 << 21), ncorr, want_ccm, nbytes);
   }
   if ( !ok ) rc = pm_fail(KINC_SIM_ENOMEM, "cannot allocate the runner's buffers");

   /* enqueue block [start, start+size) into slot s: compute, compact, counts and status to the host */
   auto launch = [&](RunSlot& s, bool compute) -> int {
      int r = KINC_SIM_OK;
      if ( compute && (r = kinc_sim_execute_block_device(ctx, s.start, s.size, s.dK, s.dL, s.dC, st)) )
         return pm_fail(r, "%s", kinc_sim_last_error(ctx));
      r = kinc_sim_compact_block_device(ctx, s.start, s.size, s.dK, s.dL, s.dC, s.dCx, s.dCy, s.dCc, s.dCr, s.cap,
                                        s.dMx, s.dMy, s.dMc, s.dMp, want_ccm ? s.cap : 0, s.dCount, st);
      if ( r ) return pm_fail(r, "%s", kinc_sim_last_error(ctx));
      if ( kinc_sim_status_copy_async(ctx, s.dCount + 2, st) != KINC_SIM_OK
           || cudaMemcpyAsync(s.hCount, s.dCount, 3 * sizeof(uint64_t), cudaMemcpyDeviceToHost, st) != cudaSuccess
           || cudaEventRecord(s.counted, st) != cudaSuccess )
         return pm_fail(KINC_SIM_ECUDA, "cannot enqueue the block's counts");
      return KINC_SIM_OK;
   };

   /* wait for slot s's counts, copy its items back on the copy stream and append them to the files */
   auto drain = [&](RunSlot& s) -> int {
      if ( cudaEventSynchronize(s.counted) != cudaSuccess )
         return pm_fail(KINC_SIM_ECUDA, "device block failed: %s", cudaGetErrorString(cudaGetLastError()));
      if ( s.hCount[2] != 0 )
      {
         const int r = kinc_sim_synchronize(ctx);
         return pm_fail(r ? r : KINC_SIM_EKERNEL, "%s", kinc_sim_last_error(ctx));
      }
      int64_t need = (int64_t)std::max(s.hCount[0], want_ccm ? s.hCount[1] : 0);
      if ( need > s.cap )
      {
         /* more kept items than the slot holds: grow it and compact this block again */
         if ( cudaStreamSynchronize(st) != cudaSuccess ) return pm_fail(KINC_SIM_ECUDA, "device block failed");
         if ( !s.alloc_items(need, ncorr, want_ccm, nbytes) )
            return pm_fail(KINC_SIM_ENOMEM, "cannot grow the item buffers to %lld", (long long)need);
         int r = launch(s, false);
         if ( r ) return r;
         if ( cudaEventSynchronize(s.counted) != cudaSuccess ) return pm_fail(KINC_SIM_ECUDA, "compaction failed");
      }
      const int64_t n_cmx = (int64_t)s.hCount[0], n_ccm = want_ccm ? (int64_t)s.hCount[1] : 0;
      bool good = cudaStreamWaitEvent(cs, s.counted, 0) == cudaSuccess;
      if ( good && ccm && n_ccm > 0 )
         good = cudaMemcpyAsync(s.hMx, s.dMx, n_ccm * 4, cudaMemcpyDeviceToHost, cs) == cudaSuccess
                && cudaMemcpyAsync(s.hMy, s.dMy, n_ccm * 4, cudaMemcpyDeviceToHost, cs) == cudaSuccess
                && cudaMemcpyAsync(s.hMc, s.dMc, n_ccm, cudaMemcpyDeviceToHost, cs) == cudaSuccess
                && cudaMemcpyAsync(s.hMp, s.dMp, (size_t)n_ccm * nbytes, cudaMemcpyDeviceToHost, cs) == cudaSuccess;
      if ( good && cmx && n_cmx > 0 )
         good = cudaMemcpyAsync(s.hCx, s.dCx, n_cmx * 4, cudaMemcpyDeviceToHost, cs) == cudaSuccess
                && cudaMemcpyAsync(s.hCy, s.dCy, n_cmx * 4, cudaMemcpyDeviceToHost, cs) == cudaSuccess
                && cudaMemcpyAsync(s.hCc, s.dCc, n_cmx, cudaMemcpyDeviceToHost, cs) == cudaSuccess
                && cudaMemcpyAsync(s.hCr, s.dCr, n_cmx * 4 * ncorr, cudaMemcpyDeviceToHost, cs) == cudaSuccess;
      if ( !good || cudaStreamSynchronize(cs) != cudaSuccess )
         return pm_fail(KINC_SIM_ECUDA, "copy of the kept items failed");
      int r = KINC_SIM_OK;
      if ( ccm && n_ccm > 0 && (r = kinc_pm_write_items_packed(ccm, n_ccm, s.hMx, s.hMy, s.hMc, s.hMp)) ) return r;
      if ( cmx && n_cmx > 0 && (r = kinc_pm_write_items(cmx, n_cmx, s.hCx, s.hCy, s.hCc, s.hCr)) ) return r;
      return KINC_SIM_OK;
   };

   const int64_t nblk = pair1 > pair0 ? (pair1 - pair0 + Bn - 1) / Bn : 0;
   for ( int64_t b = 0; rc == KINC_SIM_OK && b <= nblk; ++b )
   {
      if ( b < nblk )
      {
         RunSlot& s = slot[b & 1];
         s.start = pair0 + b * Bn;
         s.size = std::min<int64_t>(Bn, pair1 - s.start);
         rc = launch(s, true);
      }
      if ( rc == KINC_SIM_OK && b > 0 ) rc = drain(slot[(b - 1) & 1]);
   }
   if ( st ) cudaStreamSynchronize(st);
   if ( cs ) cudaStreamSynchronize(cs);
   slot[0].release();
   slot[1].release();
   if ( st ) cudaStreamDestroy(st);
   if ( cs ) cudaStreamDestroy(cs);
   const int rc1 = ccm ? kinc_pm_close(ccm) : KINC_SIM_OK;
   const int rc2 = cmx ? kinc_pm_close(cmx) : KINC_SIM_OK;
   return rc ? rc : (rc1 ? rc1 : rc2);
}
