/*
 * hnsw_oracle.c -- CPU restatement of hnsw-engine's batched query path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle the GPU library is
 * checked against.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg load it; the shipped library never links, calls or falls back
 * to it.
 *
 * Parity pin: every function below is checked against outputs of the
 * reference itself (graphs it built and saved, search_batch / brute-force
 * results it returned) committed as fixtures under tests/golden/ together
 * with the script that produced them.
 *
 * What is restated (reference paths are relative to the hnsw-engine repo):
 *   - FORMAT v1 loading and validation      src/persist.cpp:125-174, 245-365, 476-541
 *   - distance kernels, per-ISA summation   src/kernels_scalar.cpp:9-22,
 *     order (scalar / AVX2 / AVX-512 /      src/kernels_avx2.cpp:11-69,
 *     NEON), so float results are bitwise   src/kernels_avx512.cpp:10-58,
 *     those of the reference on that host   src/kernels_neon.cpp:10-54
 *   - Space / prepare_vector                src/space.hpp:23-40
 *   - greedy_closest, search_layer (Alg.2)  src/search_layer.cpp:29-134
 *   - search_unlocked / search / batch      src/search_layer.cpp:146-194
 *   - eligibility, BitsetFilter             src/index_impl.hpp:259-261,
 *                                           include/hnsw/filter.hpp:39-41
 *   - mark_deleted                          src/index.cpp:308-318
 *   - BruteForceIndex::search(_batch)       src/brute_force.cpp:34-69
 *   - parallel_for work sharing             src/threadpool.cpp:18-52
 *
 * Compile with -ffp-contract=off: every fused multiply-add below is an
 * explicit fmaf(), every other product/sum is rounded separately, exactly as
 * the reference's kernels do.
 */
#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#define ORC_API __attribute__((visibility("default")))

enum { ORC_L2 = 0, ORC_IP = 1, ORC_COSINE = 2 };
enum { ORC_SCALAR = 0, ORC_AVX2 = 1, ORC_AVX512 = 2, ORC_NEON = 3 };

#define KNONODE 0xFFFFFFFFu
#define KMAXLEVEL 64
#define KHEADER 256
#define KALIGN 64
#define KPAD 16
#define INVALID_LABEL (~(uint64_t)0)

/* ------------------------------------------------------------------------ */
/* Distance kernels: one function per ISA, each reproducing that ISA's      */
/* accumulator layout and horizontal-reduction order.                       */
/* ------------------------------------------------------------------------ */

/* kernels_scalar.cpp:9-22 -- sequential, product and sum rounded apart. */
static float l2_scalar(const float* a, const float* b, size_t n) {
  float s = 0.0f;
  for (size_t i = 0; i < n; ++i) {
    const float d = a[i] - b[i];
    s = s + d * d;
  }
  return s;
}
static float dot_scalar(const float* a, const float* b, size_t n) {
  float s = 0.0f;
  for (size_t i = 0; i < n; ++i) s = s + a[i] * b[i];
  return s;
}

/* kernels_avx2.cpp:11-18: hsum256 = ((v0+v4)+(v2+v6)) + ((v1+v5)+(v3+v7)). */
static float hsum8(const float v[8]) {
  const float s0 = v[0] + v[4], s1 = v[1] + v[5], s2 = v[2] + v[6], s3 = v[3] + v[7];
  const float t0 = s0 + s2, t1 = s1 + s3;
  return t0 + t1;
}

/* kernels_avx2.cpp:22-46: 4 x 8-lane accumulators over 32-blocks, 8-blocks
 * into acc0, reduce, then a scalar tail (built with -mfma: contracted). */
static float avx2_generic(const float* a, const float* b, size_t n, int l2) {
  float acc[4][8];
  memset(acc, 0, sizeof acc);
  size_t i = 0;
  for (; i + 32 <= n; i += 32)
    for (int j = 0; j < 4; ++j)
      for (int l = 0; l < 8; ++l) {
        const float x = a[i + 8 * j + l], y = b[i + 8 * j + l];
        if (l2) {
          const float d = x - y;
          acc[j][l] = fmaf(d, d, acc[j][l]);
        } else {
          acc[j][l] = fmaf(x, y, acc[j][l]);
        }
      }
  for (; i + 8 <= n; i += 8)
    for (int l = 0; l < 8; ++l) {
      const float x = a[i + l], y = b[i + l];
      if (l2) {
        const float d = x - y;
        acc[0][l] = fmaf(d, d, acc[0][l]);
      } else {
        acc[0][l] = fmaf(x, y, acc[0][l]);
      }
    }
  float v[8];
  for (int l = 0; l < 8; ++l) v[l] = (acc[0][l] + acc[1][l]) + (acc[2][l] + acc[3][l]);
  float s = hsum8(v);
  if (l2) {
    for (; i < n; ++i) {
      const float d = a[i] - b[i];
      s = fmaf(d, d, s);
    }
  } else {
    /* the reference build's dot tail: 4-wide products rounded on their own
     * and added in order, then a fused remainder (matched against its
     * outputs for every tail length) */
    for (; i + 4 <= n; i += 4)
      for (int l = 0; l < 4; ++l) {
        const float p = a[i + l] * b[i + l];
        s = s + p;
      }
    for (; i < n; ++i) s = fmaf(a[i], b[i], s);
  }
  return s;
}

/* GCC's _mm512_reduce_add_ps: halves 16->8->4, then {2,3,0,1} shuffle, then
 * the last pair: a butterfly over lane distance 8, 4, 2, 1. */
static float reduce16(const float v[16]) {
  float t8[8], t4[4];
  for (int i = 0; i < 8; ++i) t8[i] = v[8 + i] + v[i];
  for (int i = 0; i < 4; ++i) t4[i] = t8[4 + i] + t8[i];
  const float u0 = t4[0] + t4[2], u1 = t4[1] + t4[3];
  return u0 + u1;
}

/* kernels_avx512.cpp:10-58: 4 x 16-lane accumulators over 64-blocks,
 * 16-blocks into acc0, a masked tail into acc1, (acc0+acc1)+(acc2+acc3). */
static float avx512_generic(const float* a, const float* b, size_t n, int l2) {
  float acc[4][16];
  memset(acc, 0, sizeof acc);
  size_t i = 0;
  for (; i + 64 <= n; i += 64)
    for (int j = 0; j < 4; ++j)
      for (int l = 0; l < 16; ++l) {
        const float x = a[i + 16 * j + l], y = b[i + 16 * j + l];
        if (l2) {
          const float d = x - y;
          acc[j][l] = fmaf(d, d, acc[j][l]);
        } else {
          acc[j][l] = fmaf(x, y, acc[j][l]);
        }
      }
  for (; i + 16 <= n; i += 16)
    for (int l = 0; l < 16; ++l) {
      const float x = a[i + l], y = b[i + l];
      if (l2) {
        const float d = x - y;
        acc[0][l] = fmaf(d, d, acc[0][l]);
      } else {
        acc[0][l] = fmaf(x, y, acc[0][l]);
      }
    }
  if (i < n) {
    /* masked load: inactive lanes read 0.0f */
    for (int l = 0; l < 16; ++l) {
      const int live = (size_t)l < n - i;
      const float x = live ? a[i + l] : 0.0f, y = live ? b[i + l] : 0.0f;
      if (l2) {
        const float d = x - y;
        acc[1][l] = fmaf(d, d, acc[1][l]);
      } else {
        acc[1][l] = fmaf(x, y, acc[1][l]);
      }
    }
  }
  float v[16];
  for (int l = 0; l < 16; ++l) v[l] = (acc[0][l] + acc[1][l]) + (acc[2][l] + acc[3][l]);
  return reduce16(v);
}

/* kernels_neon.cpp:10-54: 4 x 4-lane accumulators over 16-blocks, 4-blocks
 * into acc0, vaddvq_f32 = (v0+v1)+(v2+v3), then a fused scalar tail. */
static float neon_generic(const float* a, const float* b, size_t n, int l2) {
  float acc[4][4];
  memset(acc, 0, sizeof acc);
  size_t i = 0;
  for (; i + 16 <= n; i += 16)
    for (int j = 0; j < 4; ++j)
      for (int l = 0; l < 4; ++l) {
        const float x = a[i + 4 * j + l], y = b[i + 4 * j + l];
        if (l2) {
          const float d = x - y;
          acc[j][l] = fmaf(d, d, acc[j][l]);
        } else {
          acc[j][l] = fmaf(x, y, acc[j][l]);
        }
      }
  for (; i + 4 <= n; i += 4)
    for (int l = 0; l < 4; ++l) {
      const float x = a[i + l], y = b[i + l];
      if (l2) {
        const float d = x - y;
        acc[0][l] = fmaf(d, d, acc[0][l]);
      } else {
        acc[0][l] = fmaf(x, y, acc[0][l]);
      }
    }
  float v[4];
  for (int l = 0; l < 4; ++l) v[l] = (acc[0][l] + acc[1][l]) + (acc[2][l] + acc[3][l]);
  float s = (v[0] + v[1]) + (v[2] + v[3]);
  for (; i < n; ++i) {
    if (l2) {
      const float d = a[i] - b[i];
      s = fmaf(d, d, s);
    } else {
      s = fmaf(a[i], b[i], s);
    }
  }
  return s;
}

static float l2_avx2(const float* a, const float* b, size_t n) { return avx2_generic(a, b, n, 1); }
static float dot_avx2(const float* a, const float* b, size_t n) { return avx2_generic(a, b, n, 0); }
static float l2_avx512(const float* a, const float* b, size_t n) { return avx512_generic(a, b, n, 1); }
static float dot_avx512(const float* a, const float* b, size_t n) { return avx512_generic(a, b, n, 0); }
static float l2_neon(const float* a, const float* b, size_t n) { return neon_generic(a, b, n, 1); }
static float dot_neon(const float* a, const float* b, size_t n) { return neon_generic(a, b, n, 0); }

typedef float (*dist_fn)(const float*, const float*, size_t);

static dist_fn kernel_for(int isa, int metric) {
  const int l2 = metric == ORC_L2;
  switch (isa) {
    case ORC_AVX2: return l2 ? l2_avx2 : dot_avx2;
    case ORC_AVX512: return l2 ? l2_avx512 : dot_avx512;
    case ORC_NEON: return l2 ? l2_neon : dot_neon;
    default: return l2 ? l2_scalar : dot_scalar;
  }
}

/* space.hpp:23-26: squared L2, or 1 - dot for inner product and cosine. */
static inline float space_dist(dist_fn k, int metric, const float* a, const float* b, size_t n) {
  const float r = k(a, b, n);
  return metric == ORC_L2 ? r : 1.0f - r;
}

/* space.hpp:31-40 */
ORC_API void orc_prepare_vector(int metric, const float* src, float* dst, size_t dim) {
  if (metric != ORC_COSINE) {
    for (size_t i = 0; i < dim; ++i) dst[i] = src[i];
    return;
  }
  double norm = 0.0;
  for (size_t i = 0; i < dim; ++i) norm += (double)src[i] * (double)src[i];
  const float inv = norm > 0.0 ? (float)(1.0 / sqrt(norm)) : 1.0f;
  for (size_t i = 0; i < dim; ++i) dst[i] = src[i] * inv;
}

ORC_API float orc_distance(int isa, int metric, const float* a, const float* b, size_t n) {
  return space_dist(kernel_for(isa, metric), metric, a, b, n);
}

ORC_API float orc_kernel(int isa, int l2, const float* a, const float* b, size_t n) {
  return kernel_for(isa, l2 ? ORC_L2 : ORC_IP)(a, b, n);
}

/* ------------------------------------------------------------------------ */
/* Loaded index                                                              */
/* ------------------------------------------------------------------------ */

typedef struct {
  uint64_t dim, pd, M, M0, count, ef_search, ef_construction, seed, max_elements;
  uint64_t upper_used, num_deleted, rng_state;
  int metric, max_level;
  uint32_t entry;
  unsigned char* file; /* whole file, sections point into it */
  size_t file_size;
  const float* vecs;
  const uint32_t* l0;
  const uint32_t* upper;
  const uint64_t* labels;
  const uint8_t* levels;
  uint8_t* deleted; /* owned copy */
  uint64_t* upper_off;
  uint64_t* lm_keys; /* label -> id open addressing */
  uint32_t* lm_vals;
  uint64_t lm_mask;
  int isa;
} orc_index;

static uint64_t fnv1a(const unsigned char* p, size_t n) {
  uint64_t h = 0xcbf29ce484222325ULL;
  for (size_t i = 0; i < n; ++i) {
    h ^= p[i];
    h *= 0x100000001b3ULL;
  }
  return h;
}

/* persist.cpp:156-174 */
typedef struct { uint64_t h; } phash;
static void ph_mix(phash* s, uint64_t w) {
  s->h ^= w * 0x9E3779B97F4A7C15ULL;
  s->h = (s->h << 31) | (s->h >> 33);
  s->h *= 0xC2B2AE3D27D4EB4FULL;
}
static void ph_update(phash* s, const unsigned char* p, size_t n) {
  size_t i = 0;
  for (; i + 8 <= n; i += 8) {
    uint64_t w;
    memcpy(&w, p + i, 8);
    ph_mix(s, w);
  }
  for (; i < n; ++i) ph_mix(s, 0x100ULL | p[i]);
  ph_mix(s, (uint64_t)n);
}

static uint64_t rd64(const unsigned char* b, size_t at) { uint64_t v; memcpy(&v, b + at, 8); return v; }
static uint32_t rd32(const unsigned char* b, size_t at) { uint32_t v; memcpy(&v, b + at, 4); return v; }

static size_t align_up64(size_t v) { return (v + KALIGN - 1) / KALIGN * KALIGN; }

static int fail(char* err, size_t errlen, const char* path, const char* why) {
  if (err && errlen) snprintf(err, errlen, "corrupt or incompatible index file '%s': %s", path, why);
  return -1;
}

static uint64_t mix64(uint64_t x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdULL;
  x ^= x >> 33;
  return x;
}

static long lm_find(const orc_index* ix, uint64_t label) {
  if (!ix->lm_keys) return -1;
  uint64_t p = mix64(label) & ix->lm_mask;
  for (;;) {
    if (ix->lm_vals[p] == KNONODE) return -1;
    if (ix->lm_keys[p] == label) return (long)ix->lm_vals[p];
    p = (p + 1) & ix->lm_mask;
  }
}

ORC_API void orc_free(orc_index* ix) {
  if (!ix) return;
  free(ix->file);
  free(ix->deleted);
  free(ix->upper_off);
  free(ix->lm_keys);
  free(ix->lm_vals);
  free(ix);
}

/* persist.cpp:245-365 and 476-541: header decode, layout, zero padding,
 * payload hash, then graph validation.  Any failure -> NULL + message. */
ORC_API orc_index* orc_load(const char* path, char* err, size_t errlen) {
  FILE* f = fopen(path, "rb");
  if (!f) {
    if (err && errlen) snprintf(err, errlen, "cannot open %s", path);
    return NULL;
  }
  fseek(f, 0, SEEK_END);
  const long sz = ftell(f);
  fseek(f, 0, SEEK_SET);
  if (sz < 0) {
    fclose(f);
    if (err && errlen) snprintf(err, errlen, "cannot stat %s", path);
    return NULL;
  }
  unsigned char* buf = (unsigned char*)malloc((size_t)sz + 1);
  if ((size_t)sz && fread(buf, 1, (size_t)sz, f) != (size_t)sz) {
    fclose(f);
    free(buf);
    if (err && errlen) snprintf(err, errlen, "short read %s", path);
    return NULL;
  }
  fclose(f);
  const size_t actual = (size_t)sz;
  orc_index* ix = (orc_index*)calloc(1, sizeof *ix);
  ix->file = buf;
  ix->file_size = actual;
  ix->isa = ORC_AVX512;
#define BAD(why) do { fail(err, errlen, path, why); orc_free(ix); return NULL; } while (0)
  if (actual < KHEADER) BAD("file too small for header");
  static const char magic[8] = {'H', 'N', 'S', 'W', 'E', 'N', 'G', '\0'};
  if (memcmp(buf, magic, 8) != 0) BAD("bad magic");
  if (rd32(buf, 12) != 0x01020304u) BAD("endianness mismatch");
  if (rd32(buf, 8) != 1u) BAD("unsupported version");
  {
    unsigned char tmp[KHEADER];
    memcpy(tmp, buf, KHEADER);
    memset(tmp + 184, 0, 8);
    if (rd64(buf, 184) != fnv1a(tmp, KHEADER)) BAD("header checksum mismatch");
  }
  ix->dim = rd64(buf, 16);
  const uint32_t metric = rd32(buf, 24);
  ix->M = rd64(buf, 32);
  ix->ef_construction = rd64(buf, 40);
  ix->ef_search = rd64(buf, 48);
  ix->seed = rd64(buf, 56);
  ix->max_elements = rd64(buf, 64);
  ix->count = rd64(buf, 72);
  ix->pd = rd64(buf, 80);
  int32_t max_level;
  memcpy(&max_level, buf + 88, 4);
  ix->max_level = max_level;
  ix->entry = rd32(buf, 92);
  ix->upper_used = rd64(buf, 96);
  ix->num_deleted = rd64(buf, 104);
  ix->rng_state = rd64(buf, 112);
  const uint64_t off_vec = rd64(buf, 120), off_l0 = rd64(buf, 128), off_lab = rd64(buf, 136),
                 off_lev = rd64(buf, 144), off_del = rd64(buf, 152), off_up = rd64(buf, 160),
                 file_size = rd64(buf, 168), payload = rd64(buf, 176);
  if (file_size != actual) BAD("size mismatch (truncated or extended file)");
  if (ix->dim == 0 || ix->dim > (1u << 20)) BAD("invalid dim");
  if (metric > 2) BAD("invalid metric");
  ix->metric = (int)metric;
  if (ix->M < 2 || ix->M > 2048) BAD("invalid M");
  if (ix->ef_construction == 0 || ix->ef_search == 0) BAD("invalid ef");
  if (ix->pd != (ix->dim + KPAD - 1) / KPAD * KPAD) BAD("invalid padded dim");
  if (ix->count > actual || ix->count >= KNONODE) BAD("invalid count");
  if (ix->upper_used > actual) BAD("invalid upper size");
  if (ix->num_deleted > ix->count) BAD("invalid deleted count");
  if (ix->max_elements != 0 && (ix->max_elements < ix->count || ix->max_elements >= KNONODE))
    BAD("invalid max_elements");
  if (ix->count == 0) {
    if (ix->max_level != -1 || ix->entry != KNONODE) BAD("invalid empty-index header");
  } else if (ix->max_level < 0 || ix->max_level > KMAXLEVEL || ix->entry >= ix->count) {
    BAD("invalid entry point / max level");
  }
  const uint64_t n = ix->count;
  ix->M0 = 2 * ix->M;
  const size_t sz_vec = n * ix->pd * 4, sz_l0 = n * (1 + ix->M0) * 4, sz_lab = n * 8, sz_lev = n,
               sz_del = n, sz_up = ix->upper_used * 4;
  size_t pos = KHEADER;
  const size_t e_vec = pos;
  pos = align_up64(pos + sz_vec);
  const size_t e_l0 = pos;
  pos = align_up64(pos + sz_l0);
  const size_t e_lab = pos;
  pos = align_up64(pos + sz_lab);
  const size_t e_lev = pos;
  pos = align_up64(pos + sz_lev);
  const size_t e_del = pos;
  pos = align_up64(pos + sz_del);
  const size_t e_up = pos;
  pos += sz_up;
  if (e_vec != off_vec || e_l0 != off_l0 || e_lab != off_lab || e_lev != off_lev || e_del != off_del ||
      e_up != off_up || pos != file_size)
    BAD("section offsets inconsistent with header");
  {
    const size_t offs[6] = {e_vec, e_l0, e_lab, e_lev, e_del, e_up};
    const size_t lens[6] = {sz_vec, sz_l0, sz_lab, sz_lev, sz_del, sz_up};
    phash h = {0x243F6A8885A308D3ULL};
    size_t p = KHEADER;
    for (int s = 0; s < 6; ++s) {
      for (size_t i = p; i < offs[s]; ++i)
        if (buf[i] != 0) BAD("non-zero padding");
      ph_update(&h, buf + offs[s], lens[s]);
      p = offs[s] + lens[s];
    }
    if (h.h != payload) BAD("payload checksum mismatch");
  }
  ix->vecs = (const float*)(buf + e_vec);
  ix->l0 = (const uint32_t*)(buf + e_l0);
  ix->labels = (const uint64_t*)(buf + e_lab);
  ix->levels = buf + e_lev;
  ix->upper = (const uint32_t*)(buf + e_up);
  /* validate_and_index, persist.cpp:321-365 */
  ix->upper_off = (uint64_t*)calloc(n ? n : 1, 8);
  uint64_t up = 0;
  const uint64_t ustride = 1 + ix->M;
  for (uint64_t i = 0; i < n; ++i) {
    const int lv = ix->levels[i];
    if (lv > ix->max_level) BAD("node level exceeds max level");
    ix->upper_off[i] = up;
    up += (uint64_t)lv * ustride;
  }
  if (up != ix->upper_used) BAD("upper-layer size does not match levels");
  if (n > 0 && ix->levels[ix->entry] != ix->max_level) BAD("entry point is not on the top level");
  for (uint64_t i = 0; i < n; ++i) {
    for (int lc = 0; lc <= ix->levels[i]; ++lc) {
      const uint32_t* l = lc == 0 ? ix->l0 + i * (1 + ix->M0) : ix->upper + ix->upper_off[i] + (uint64_t)(lc - 1) * ustride;
      if (l[0] > (lc == 0 ? ix->M0 : ix->M)) BAD("neighbor count exceeds maximum degree");
      for (uint32_t j = 0; j < l[0]; ++j) {
        const uint32_t nb = l[1 + j];
        if (nb >= n || ix->levels[nb] < lc) BAD("neighbor id out of range");
      }
    }
  }
  uint64_t cap = 16;
  while (cap < 2 * n) cap <<= 1;
  ix->lm_mask = cap - 1;
  ix->lm_keys = (uint64_t*)calloc(cap, 8);
  ix->lm_vals = (uint32_t*)malloc(cap * 4);
  memset(ix->lm_vals, 0xFF, cap * 4);
  for (uint64_t i = 0; i < n; ++i) {
    const uint64_t lab = ix->labels[i];
    uint64_t p = mix64(lab) & ix->lm_mask;
    for (;;) {
      if (ix->lm_vals[p] == KNONODE) {
        ix->lm_keys[p] = lab;
        ix->lm_vals[p] = (uint32_t)i;
        break;
      }
      if (ix->lm_keys[p] == lab) BAD("duplicate label");
      p = (p + 1) & ix->lm_mask;
    }
  }
  ix->deleted = (uint8_t*)malloc(n ? n : 1);
  memcpy(ix->deleted, buf + e_del, n);
  uint64_t dels = 0;
  for (uint64_t i = 0; i < n; ++i) {
    if (ix->deleted[i] > 1) BAD("invalid tombstone byte");
    dels += ix->deleted[i];
  }
  if (dels != ix->num_deleted) BAD("deleted count mismatch");
#undef BAD
  return ix;
}

typedef struct {
  uint64_t dim, pd, M, count, ef_search, num_deleted;
  int64_t metric, max_level, entry;
} orc_info_t;

ORC_API void orc_info(const orc_index* ix, orc_info_t* out) {
  out->dim = ix->dim;
  out->pd = ix->pd;
  out->M = ix->M;
  out->count = ix->count;
  out->ef_search = ix->ef_search;
  out->num_deleted = ix->num_deleted;
  out->metric = ix->metric;
  out->max_level = ix->max_level;
  out->entry = ix->entry == KNONODE ? -1 : (int64_t)ix->entry;
}

ORC_API void orc_set_isa(orc_index* ix, int isa) { ix->isa = isa; }
ORC_API void orc_set_ef(orc_index* ix, uint64_t ef) { ix->ef_search = ef; }

/* index.cpp:308-318.  Returns 0, or -1 for an unknown label. */
ORC_API int orc_mark_deleted(orc_index* ix, uint64_t label) {
  const long id = lm_find(ix, label);
  if (id < 0) return -1;
  if (ix->deleted[id] == 0) {
    ix->deleted[id] = 1;
    ++ix->num_deleted;
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Search (search_layer.cpp)                                                 */
/* ------------------------------------------------------------------------ */

typedef struct { float d; uint32_t id; } cand_t;

/* index_impl.hpp:58-71: total order on (dist, internal id). */
static inline int cless(cand_t a, cand_t b) { return a.d < b.d || (a.d == b.d && a.id < b.id); }

/* Binary heaps.  With unique ids the order is total, so any correct heap
 * pops exactly what std::push_heap/pop_heap pop in the reference. */
typedef struct { cand_t* a; size_t n, cap; } heap_t;

static void heap_reserve(heap_t* h, size_t need) {
  if (need <= h->cap) return;
  size_t c = h->cap ? h->cap : 64;
  while (c < need) c *= 2;
  h->a = (cand_t*)realloc(h->a, c * sizeof(cand_t));
  h->cap = c;
}
/* max-heap by cless (res) when maxh = 1, min-heap (cand) when maxh = 0 */
static inline int hbefore(cand_t x, cand_t y, int maxh) { return maxh ? cless(y, x) : cless(x, y); }
static void heap_push(heap_t* h, cand_t x, int maxh) {
  heap_reserve(h, h->n + 1);
  size_t i = h->n++;
  while (i > 0) {
    const size_t p = (i - 1) / 2;
    if (!hbefore(x, h->a[p], maxh)) break;
    h->a[i] = h->a[p];
    i = p;
  }
  h->a[i] = x;
}
static cand_t heap_pop(heap_t* h, int maxh) {
  const cand_t top = h->a[0];
  const cand_t x = h->a[--h->n];
  size_t i = 0;
  for (;;) {
    size_t c = 2 * i + 1;
    if (c >= h->n) break;
    if (c + 1 < h->n && hbefore(h->a[c + 1], h->a[c], maxh)) ++c;
    if (!hbefore(h->a[c], x, maxh)) break;
    h->a[i] = h->a[c];
    i = c;
  }
  if (h->n > 0) h->a[i] = x;
  return top;
}

typedef struct {
  uint32_t* marks;
  uint32_t epoch;
  size_t marks_n;
  heap_t cand, res;
  float* query;
} scratch_t;

static void scratch_free(scratch_t* s) {
  free(s->marks);
  free(s->cand.a);
  free(s->res.a);
  free(s->query);
}

/* Per-query traversal counts, the inputs of the algorithmic-byte figure. */
enum { CNT_UP_LISTS = 0, CNT_UP_DISTS, CNT_L0_LISTS, CNT_L0_DISTS, CNT_VISITED, CNT_MAX_CAND, CNT_RES, CNT_N };

typedef struct {
  const uint64_t* words;
  uint64_t size_bits;
  int active;
} filter_t;

static inline int allowed(const filter_t* f, uint64_t label) {
  return label < f->size_bits && ((f->words[label >> 6] >> (label & 63)) & 1ULL) != 0;
}

/* index_impl.hpp:259-261 */
static inline int eligible(const orc_index* ix, uint32_t id, const filter_t* f) {
  return ix->deleted[id] == 0 && (!f->active || allowed(f, ix->labels[id]));
}

static inline const float* vec(const orc_index* ix, uint32_t id) { return ix->vecs + (uint64_t)id * ix->pd; }
static inline const uint32_t* list_at(const orc_index* ix, uint32_t id, int level) {
  return level == 0 ? ix->l0 + (uint64_t)id * (1 + ix->M0)
                    : ix->upper + ix->upper_off[id] + (uint64_t)(level - 1) * (1 + ix->M);
}

/* search_layer.cpp:29-56 (Locked = false) */
static cand_t greedy_closest(const orc_index* ix, dist_fn k, const float* q, cand_t cur, int level, uint64_t* cnt) {
  int changed = 1;
  while (changed) {
    changed = 0;
    const uint32_t* l = list_at(ix, cur.id, level);
    const uint32_t n = l[0];
    cnt[CNT_UP_LISTS]++;
    for (uint32_t j = 0; j < n; ++j) {
      const float d = space_dist(k, ix->metric, q, vec(ix, l[1 + j]), ix->pd);
      cnt[CNT_UP_DISTS]++;
      if (d < cur.d) {
        cur.d = d;
        cur.id = l[1 + j];
        changed = 1;
      }
    }
  }
  return cur;
}

/* search_layer.cpp:58-134 (Locked = false), one entry point, level 0. */
static void search_layer0(const orc_index* ix, dist_fn k, const float* q, cand_t ep, size_t ef, int filtered,
                          const filter_t* f, scratch_t* s, uint64_t* cnt) {
  if (s->marks_n < ix->count) {
    free(s->marks);
    s->marks = (uint32_t*)calloc(ix->count ? ix->count : 1, 4);
    s->marks_n = ix->count;
    s->epoch = 0;
  }
  if (++s->epoch == 0) {
    memset(s->marks, 0, s->marks_n * 4);
    s->epoch = 1;
  }
  heap_t* cand = &s->cand;
  heap_t* res = &s->res;
  cand->n = 0;
  res->n = 0;
  s->marks[ep.id] = s->epoch;
  cnt[CNT_VISITED]++;
  heap_push(cand, ep, 0);
  if (!filtered || eligible(ix, ep.id, f)) heap_push(res, ep, 1);
  while (res->n > ef) heap_pop(res, 1);
  while (cand->n > 0) {
    if (cand->n > cnt[CNT_MAX_CAND]) cnt[CNT_MAX_CAND] = cand->n;
    const cand_t c = cand->a[0];
    if (res->n >= ef && c.d > res->a[0].d) break;
    heap_pop(cand, 0);
    const uint32_t* l = list_at(ix, c.id, 0);
    const uint32_t n = l[0];
    cnt[CNT_L0_LISTS]++;
    for (uint32_t j = 0; j < n; ++j) {
      const uint32_t id = l[1 + j];
      if (s->marks[id] == s->epoch) continue;
      s->marks[id] = s->epoch;
      cnt[CNT_VISITED]++;
      const float d = space_dist(k, ix->metric, q, vec(ix, id), ix->pd);
      cnt[CNT_L0_DISTS]++;
      if (res->n < ef || d < res->a[0].d) {
        const cand_t x = {d, id};
        heap_push(cand, x, 0);
        if (!filtered || eligible(ix, id, f)) {
          heap_push(res, x, 1);
          if (res->n > ef) heap_pop(res, 1);
        }
      }
    }
  }
}

static int cmp_cand(const void* a, const void* b) {
  const cand_t x = *(const cand_t*)a, y = *(const cand_t*)b;
  return cless(x, y) ? -1 : (cless(y, x) ? 1 : 0);
}

/* search_layer.cpp:146-171.  Returns the number of results written. */
static size_t search_one(const orc_index* ix, const float* qraw, size_t k, size_t ef, const filter_t* f, scratch_t* s,
                         uint64_t* labels_out, float* dists_out, uint64_t* cnt) {
  if (ix->count == 0) return 0;
  ef = ef == 0 ? ix->ef_search : ef;
  if (ef < k) ef = k;
  if (!s->query) s->query = (float*)calloc(ix->pd, 4);
  orc_prepare_vector(ix->metric, qraw, s->query, ix->dim);
  const dist_fn kern = kernel_for(ix->isa, ix->metric);
  const float* q = s->query;
  cand_t cur = {space_dist(kern, ix->metric, q, vec(ix, ix->entry), ix->pd), ix->entry};
  cnt[CNT_UP_DISTS]++;
  for (int lc = ix->max_level; lc > 0; --lc) cur = greedy_closest(ix, kern, q, cur, lc, cnt);
  const int filtered = f->active || ix->num_deleted > 0;
  search_layer0(ix, kern, q, cur, ef, filtered, f, s, cnt);
  heap_t* res = &s->res;
  qsort(res->a, res->n, sizeof(cand_t), cmp_cand);
  cnt[CNT_RES] = res->n;
  const size_t m = k < res->n ? k : res->n;
  for (size_t i = 0; i < m; ++i) {
    labels_out[i] = ix->labels[res->a[i].id];
    dists_out[i] = res->a[i].d;
  }
  return m;
}

typedef struct {
  const orc_index* ix;
  const float* qs;
  size_t nq, k, dim;
  const size_t* ef;  /* per query */
  const size_t* kq;  /* per query k (<= k), NULL = k */
  const filter_t* filters;
  const int32_t* fsel; /* per query filter index, -1 = none; NULL = all use filters[0] */
  uint64_t* labels;
  float* dists;
  uint64_t* counters; /* CNT_N per query or NULL */
  atomic_size_t next;
} batch_job;

static void* batch_worker(void* arg) {
  batch_job* J = (batch_job*)arg;
  scratch_t s;
  memset(&s, 0, sizeof s);
  const filter_t nofilter = {NULL, 0, 0};
  for (;;) {
    const size_t i = atomic_fetch_add(&J->next, 1);
    if (i >= J->nq) break;
    uint64_t cnt[CNT_N] = {0};
    const filter_t* f = &nofilter;
    if (J->filters) {
      if (J->fsel == NULL) f = &J->filters[0];
      else if (J->fsel[i] >= 0) f = &J->filters[J->fsel[i]];
    }
    const size_t kq = J->kq ? J->kq[i] : J->k;
    uint64_t* lrow = J->labels + i * J->k;
    float* drow = J->dists + i * J->k;
    const size_t m = search_one(J->ix, J->qs + i * J->dim, kq, J->ef[i], f, &s, lrow, drow, cnt);
    for (size_t j = m; j < J->k; ++j) {
      lrow[j] = INVALID_LABEL;
      drow[j] = INFINITY;
    }
    if (J->counters) memcpy(J->counters + i * CNT_N, cnt, sizeof cnt);
  }
  scratch_free(&s);
  return NULL;
}

static size_t resolve_threads(size_t t) {
  if (t) return t;
  const long hw = sysconf(_SC_NPROCESSORS_ONLN);
  return hw > 0 ? (size_t)hw : 1;
}

static void run_batch(batch_job* J, size_t nthreads) {
  atomic_store(&J->next, 0);
  size_t w = resolve_threads(nthreads);
  if (w > J->nq) w = J->nq;
  if (w <= 1) {
    batch_worker(J);
    return;
  }
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * w);
  for (size_t t = 1; t < w; ++t) pthread_create(&th[t], NULL, batch_worker, J);
  batch_worker(J);
  for (size_t t = 1; t < w; ++t) pthread_join(th[t], NULL);
  free(th);
}

/* Index::search_batch, search_layer.cpp:180-194, generalised to per-query
 * ef / k / filter selection (each group equals one reference call).
 * labels/dists: nq*k, padded with {INVALID_LABEL, +inf}.  ef_per_query may
 * be NULL (then ef applies to all).  filter_words/sizes: nfilters bitsets by
 * label; fsel per query (-1 none) or NULL (filter 0 for all, if any). */
ORC_API int orc_search_batch(const orc_index* ix, const float* qs, size_t nq, size_t k, size_t ef,
                             const uint64_t* ef_per_query, const uint64_t* k_per_query,
                             const uint64_t* const* filter_words, const uint64_t* filter_sizes, size_t nfilters,
                             const int32_t* fsel, uint64_t* labels, float* dists, uint64_t* counters,
                             size_t nthreads) {
  if (k == 0 || nq == 0) return k == 0 ? -1 : 0;
  size_t* efs = (size_t*)malloc(nq * sizeof(size_t));
  size_t* ks = k_per_query ? (size_t*)malloc(nq * sizeof(size_t)) : NULL;
  for (size_t i = 0; i < nq; ++i) {
    efs[i] = ef_per_query ? (size_t)ef_per_query[i] : ef;
    if (ks) ks[i] = (size_t)k_per_query[i];
  }
  filter_t* fl = NULL;
  if (nfilters) {
    fl = (filter_t*)malloc(nfilters * sizeof(filter_t));
    for (size_t i = 0; i < nfilters; ++i) {
      fl[i].words = filter_words[i];
      fl[i].size_bits = filter_sizes[i];
      fl[i].active = 1;
    }
  }
  batch_job J;
  J.ix = ix;
  J.qs = qs;
  J.nq = nq;
  J.k = k;
  J.dim = ix->dim;
  J.ef = efs;
  J.kq = ks;
  J.filters = fl;
  J.fsel = fsel;
  J.labels = labels;
  J.dists = dists;
  J.counters = counters;
  run_batch(&J, nthreads);
  free(efs);
  free(ks);
  free(fl);
  return 0;
}

/* Index::search (search_layer.cpp:173-178): no padding; returns count. */
ORC_API long orc_search(const orc_index* ix, const float* q, size_t k, size_t ef, const uint64_t* filter_words,
                        uint64_t filter_size, int has_filter, uint64_t* labels, float* dists) {
  if (k == 0 || q == NULL) return -1;
  scratch_t s;
  memset(&s, 0, sizeof s);
  const filter_t f = {filter_words, filter_size, has_filter};
  uint64_t cnt[CNT_N] = {0};
  const size_t m = search_one(ix, q, k, ef, &f, &s, labels, dists, cnt);
  scratch_free(&s);
  return (long)m;
}

/* ------------------------------------------------------------------------ */
/* Brute force (brute_force.cpp:24-69)                                       */
/* ------------------------------------------------------------------------ */

typedef struct { uint64_t label; float d; } nb_t;

/* brute_force.cpp:15-17: (distance, label) order */
static inline int nless(nb_t a, nb_t b) { return a.d < b.d || (a.d == b.d && a.label < b.label); }

static void nheap_push(nb_t* h, size_t* n, nb_t x) {
  size_t i = (*n)++;
  while (i > 0) {
    const size_t p = (i - 1) / 2;
    if (!nless(h[p], x)) break;
    h[i] = h[p];
    i = p;
  }
  h[i] = x;
}
static void nheap_replace_top(nb_t* h, size_t n, nb_t x) {
  size_t i = 0;
  for (;;) {
    size_t c = 2 * i + 1;
    if (c >= n) break;
    if (c + 1 < n && nless(h[c], h[c + 1])) ++c;
    if (!nless(x, h[c])) break;
    h[i] = h[c];
    i = c;
  }
  h[i] = x;
}
static int cmp_nb(const void* a, const void* b) {
  const nb_t x = *(const nb_t*)a, y = *(const nb_t*)b;
  return nless(x, y) ? -1 : (nless(y, x) ? 1 : 0);
}

typedef struct {
  const float* data; /* prepared, n x dim */
  const uint64_t* labels;
  size_t n, dim, nq, k;
  int metric, isa;
  const float* qs;
  filter_t f;
  uint64_t* out_labels;
  float* out_d;
  atomic_size_t next;
} bf_job;

static void* bf_worker(void* arg) {
  bf_job* J = (bf_job*)arg;
  const dist_fn kern = kernel_for(J->isa, J->metric);
  float* q = (float*)malloc(J->dim * 4);
  nb_t* heap = (nb_t*)malloc((J->k + 1) * sizeof(nb_t));
  for (;;) {
    const size_t i = atomic_fetch_add(&J->next, 1);
    if (i >= J->nq) break;
    orc_prepare_vector(J->metric, J->qs + i * J->dim, q, J->dim);
    size_t hn = 0;
    for (size_t r = 0; r < J->n; ++r) {
      if (J->f.active && !allowed(&J->f, J->labels[r])) continue;
      const nb_t c = {J->labels[r], space_dist(kern, J->metric, q, J->data + r * J->dim, J->dim)};
      if (hn < J->k) nheap_push(heap, &hn, c);
      else if (nless(c, heap[0])) nheap_replace_top(heap, hn, c);
    }
    qsort(heap, hn, sizeof(nb_t), cmp_nb);
    for (size_t j = 0; j < J->k; ++j) {
      J->out_labels[i * J->k + j] = j < hn ? heap[j].label : INVALID_LABEL;
      J->out_d[i * J->k + j] = j < hn ? heap[j].d : INFINITY;
    }
  }
  free(q);
  free(heap);
  return NULL;
}

/* BruteForceIndex::add + search_batch.  data is raw (un-normalised); labels
 * may be NULL (then 0..n-1, as add() does). */
ORC_API int orc_bruteforce(const float* data, const uint64_t* labels, size_t n, size_t dim, int metric, int isa,
                           const float* qs, size_t nq, size_t k, const uint64_t* filter_words, uint64_t filter_size,
                           int has_filter, uint64_t* out_labels, float* out_d, size_t nthreads) {
  if (k == 0 || dim == 0) return -1;
  float* prepared = (float*)malloc((n ? n : 1) * dim * 4);
  uint64_t* labs = (uint64_t*)malloc((n ? n : 1) * 8);
  for (size_t i = 0; i < n; ++i) {
    orc_prepare_vector(metric, data + i * dim, prepared + i * dim, dim);
    labs[i] = labels ? labels[i] : (uint64_t)i;
  }
  bf_job J;
  J.data = prepared;
  J.labels = labs;
  J.n = n;
  J.dim = dim;
  J.nq = nq;
  J.k = k;
  J.metric = metric;
  J.isa = isa;
  J.qs = qs;
  J.f.words = filter_words;
  J.f.size_bits = filter_size;
  J.f.active = has_filter;
  J.out_labels = out_labels;
  J.out_d = out_d;
  atomic_store(&J.next, 0);
  size_t w = resolve_threads(nthreads);
  if (w > nq) w = nq ? nq : 1;
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * w);
  for (size_t t = 1; t < w; ++t) pthread_create(&th[t], NULL, bf_worker, &J);
  bf_worker(&J);
  for (size_t t = 1; t < w; ++t) pthread_join(th[t], NULL);
  free(th);
  free(prepared);
  free(labs);
  return 0;
}

ORC_API int orc_counter_count(void) { return CNT_N; }
