// Text I/O of the analysis path on the device: the GridObservation text
// format (GridObservation::loadFromFile, src/backends/common/observation/
// GridObservation.hpp:395-474), SimpleState files (SimpleState::readFromFile,
// src/backends/simple/SimpleState.hpp:248-263) and the state writer
// (SimpleState::saveToFile, :160-188).
//
// The text is copied to the device once; lines are indexed in parallel
// (per-4 KB chunk counts, a scan, then the line starts), and every line is
// scanned with the extraction rules of std::istream (one thread per line, or
// for long lines of values one warp per line, below):
//   * int: skip white space, optional sign, at least one digit;
//   * double: skip white space, [sign] (digits [. digits] | . digits)
//     [(e|E) [sign] digits]; no inf/nan/hex (libstdc++ rejects them);
//   * the next extraction starts right after the previous one.
// Decimal to binary, each step exact (equal to strtod):
//   * a mantissa below 2^53 with a decimal exponent in [-22, 22]: one
//     correctly rounded multiplication or division by an exact power of ten
//     (Clinger's fast path);
//   * any other mantissa of at most 19 significant digits: the Eisel-Lemire
//     algorithm (a 128-bit product with a table of powers of five), when the
//     result is a normal double;
//   * more than 19 significant digits: the first 19 (w) decide alone when
//     the dropped digits are zeros, otherwise w and w + 1 are converted and
//     the result stands when both give the same double.
// Numbers left over (subnormal or overflowing results, and the rare long
// mantissas whose two bounds round apart) send their line to the host, where
// std::istringstream (the reference's own extraction) reads it.
// The writer prints "%12.6f" values (std::fixed, setprecision(6),
// setw(12)) joined by one space, one row of x values per line: |v| < 2^53
// is rounded exactly to 6 decimals (round half to even on the binary value,
// as printf) with 128-bit integer arithmetic; other values (and NaN/inf) are
// printed on the host.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <sstream>
#include <string>
#include <vector>

#include "mg_internal.h"
#include "mg_pow5.h"

namespace {

constexpr int kThreads = 256;
constexpr int64_t kChunk = 4096;

__device__ __forceinline__ bool is_ws(char c) {
  return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r';
}
__device__ __forceinline__ bool is_digit(char c) { return c >= '0' && c <= '9'; }

// ---- line index ----
__global__ void line_count_kernel(const char* __restrict__ t, int64_t n, int64_t* __restrict__ counts) {
  const int64_t c0 = (int64_t)blockIdx.x * kChunk;
  const int64_t c1 = c0 + kChunk < n ? c0 + kChunk : n;
  __shared__ int red[kThreads / 32];
  int cnt = 0;
  for (int64_t i = c0 + threadIdx.x; i < c1; i += kThreads) cnt += (i == 0 || t[i - 1] == '\n') ? 1 : 0;
  for (int off = 16; off > 0; off >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int w = 0; w < kThreads / 32; ++w) s += red[w];
    counts[blockIdx.x] = s;
  }
}

// Line starts in text order: a chunk's threads take consecutive 16-byte
// pieces; a block-wide exclusive scan of the per-thread counts gives each
// thread's first slot.
__global__ void line_fill_kernel(const char* __restrict__ t, int64_t n, const int64_t* __restrict__ offsets,
                                 int64_t* __restrict__ starts) {
  constexpr int kPiece = (int)(kChunk / kThreads);  // 16 bytes per thread
  const int64_t c0 = (int64_t)blockIdx.x * kChunk;
  const int64_t p0 = c0 + (int64_t)threadIdx.x * kPiece;
  int cnt = 0;
  for (int j = 0; j < kPiece; ++j) {
    const int64_t i = p0 + j;
    if (i < n && (i == 0 || t[i - 1] == '\n')) ++cnt;
  }
  __shared__ int scan[kThreads];
  scan[threadIdx.x] = cnt;
  __syncthreads();
  for (int off = 1; off < kThreads; off <<= 1) {  // inclusive Hillis-Steele scan
    const int v = threadIdx.x >= off ? scan[threadIdx.x - off] : 0;
    __syncthreads();
    scan[threadIdx.x] += v;
    __syncthreads();
  }
  int64_t slot = offsets[blockIdx.x] + scan[threadIdx.x] - cnt;
  for (int j = 0; j < kPiece; ++j) {
    const int64_t i = p0 + j;
    if (i < n && (i == 0 || t[i - 1] == '\n')) starts[slot++] = i;
  }
}

// ---- std::istream-style extraction ----
__device__ bool extract_int(const char* t, int64_t& pos, int64_t end, int& out) {
  while (pos < end && is_ws(t[pos])) ++pos;
  bool neg = false;
  if (pos < end && (t[pos] == '+' || t[pos] == '-')) neg = t[pos++] == '-';
  if (pos >= end || !is_digit(t[pos])) return false;
  long long v = 0;
  while (pos < end && is_digit(t[pos])) {
    v = v * 10 + (t[pos++] - '0');
    if (v > 2147483648ll) return false;  // overflow: failbit
  }
  if (!neg && v > 2147483647ll) return false;
  out = (int)(neg ? -v : v);
  return true;
}

// 10^e, 0 <= e <= 22, exact in binary64 (a global table: a local one would
// be rebuilt on the thread's stack at every call).
__device__ const double kPow10[23] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,  1e8,  1e9,  1e10, 1e11,
                                      1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};
__device__ __forceinline__ double pow10_exact(int e) { return kPow10[e]; }

// The double nearest w * 10^q (w != 0) by the Eisel-Lemire algorithm
// (D. Lemire, "Number Parsing at a Gigabyte per Second", Software: Practice
// and Experience 51(8), 2021; N. Mushtak and D. Lemire, "Fast number parsing
// without fallback", 2023, show that the 128-bit product always decides for
// binary64): w normalised, multiplied by the table's 128-bit significand of
// 5^q (the low word only when the high product's low 9 bits are all ones),
// the top 54 bits rounded to nearest even, the binary exponent from
// floor(q log2(10)) = (217706 q) >> 16.  False when the result is not a
// normal double (the host converts those).
__device__ bool eisel_lemire(unsigned long long w, int q, unsigned long long& bits) {
  if (q < MG_POW5_QMIN || q > MG_POW5_QMAX) return false;
  const int lz = __clzll((long long)w);
  w <<= lz;
  const int idx = 2 * (q - MG_POW5_QMIN);
  const unsigned long long th = kPow5Table[idx], tl = kPow5Table[idx + 1];
  unsigned long long hi = __umul64hi(w, th), lo = w * th;
  if ((hi & 0x1FFull) == 0x1FFull) {
    const unsigned long long p2 = __umul64hi(w, tl);
    lo += p2;
    if (p2 > lo) ++hi;
  }
  const int upper = (int)(hi >> 63);
  const int shift = upper + 9;
  unsigned long long mant = hi >> shift;
  int power2 = (int)(((217706ll * q) >> 16) + 63) + upper - lz + 1023;
  if (power2 <= 0) return false;
  // an exact halfway point (nothing below the kept bits) rounds to even
  if (lo <= 1 && q >= -4 && q <= 23 && (mant & 3ull) == 1ull && (mant << shift) == hi) mant &= ~1ull;
  mant += mant & 1ull;
  mant >>= 1;
  if (mant >= (2ull << 52)) {
    mant = 1ull << 52;
    ++power2;
  }
  mant &= ~(1ull << 52);
  if (power2 >= 0x7FF) return false;
  bits = ((unsigned long long)power2 << 52) | mant;
  return true;
}

// Returns 1 on success, 0 on a failed extraction, 2 if the number is valid
// but not converted on the device (the host converts it).
__device__ int extract_double(const char* t, int64_t& pos, int64_t end, double& out) {
  while (pos < end && is_ws(t[pos])) ++pos;
  bool neg = false;
  if (pos < end && (t[pos] == '+' || t[pos] == '-')) neg = t[pos++] == '-';
  unsigned long long m = 0;
  int sig = 0, drop_int = 0, frac = 0, ndig = 0;
  bool nz_drop = false;  // a nonzero digit beyond the first 19 significant ones
  while (pos < end && is_digit(t[pos])) {
    const int d = t[pos++] - '0';
    ++ndig;
    if (sig == 0 && d == 0) continue;
    if (sig < 19) {
      m = m * 10 + d;
      ++sig;
    } else {
      ++drop_int;  // an integer digit beyond 19 significant ones scales by ten
      nz_drop |= d != 0;
    }
  }
  if (pos < end && t[pos] == '.') {
    ++pos;
    while (pos < end && is_digit(t[pos])) {
      const int d = t[pos++] - '0';
      ++ndig;
      if (sig == 0 && d == 0) {
        ++frac;
        continue;
      }
      if (sig < 19) {
        m = m * 10 + d;
        ++sig;
        ++frac;
      } else {
        nz_drop |= d != 0;  // a fractional digit beyond 19 significant ones
      }
    }
  }
  if (ndig == 0) return 0;
  int ex = 0;
  if (pos < end && (t[pos] == 'e' || t[pos] == 'E')) {
    int64_t q = pos + 1;
    bool eneg = false;
    if (q < end && (t[q] == '+' || t[q] == '-')) eneg = t[q++] == '-';
    if (q >= end || !is_digit(t[q])) return 0;  // "1e" with no exponent digits fails
    int v = 0;
    while (q < end && is_digit(t[q])) {
      if (v < 100000) v = v * 10 + (t[q] - '0');
      ++q;
    }
    ex = eneg ? -v : v;
    pos = q;
  }
  if (m == 0) {
    out = neg ? -0.0 : 0.0;
    return 1;
  }
  const int e10 = ex - frac + drop_int;
  double v;
  if (!nz_drop && m < (1ull << 53) && e10 >= -22 && e10 <= 22) {
    const double md = (double)m;  // exact
    v = e10 >= 0 ? __dmul_rn(md, pow10_exact(e10)) : __ddiv_rn(md, pow10_exact(-e10));
  } else {
    unsigned long long b0 = 0, b1 = 0;
    if (!eisel_lemire(m, e10, b0)) return 2;
    // dropped nonzero digits: the value lies strictly between m and m + 1
    // (times 10^e10), so both bounds rounding alike decide it
    if (nz_drop && (!eisel_lemire(m + 1, e10, b1) || b1 != b0)) return 2;
    v = __longlong_as_double((long long)b0);
  }
  out = neg ? -v : v;
  return 1;
}

// ---- GridObservation text ----
enum LineType : int32_t { kEmpty = 0, kHeader = 1, kSep = 2, kData = 3, kBad = 4, kHost = 5 };

__device__ bool line_contains(const char* t, int64_t s, int64_t e, const char* pat, int np) {
  for (int64_t i = s; i + np <= e; ++i) {
    int j = 0;
    while (j < np && t[i + j] == pat[j]) ++j;
    if (j == np) return true;
  }
  return false;
}

struct ObsLines {
  int32_t* type;
  int32_t* ival;   // L x 4: time, z, y, x
  double* dval;    // L x 4: znu, xlong_u, xlat_u, value
};

__global__ void obs_lines_kernel(const char* __restrict__ t, int64_t n, const int64_t* __restrict__ starts,
                                 int64_t L, ObsLines ol, unsigned long long* __restrict__ first_header,
                                 int32_t* __restrict__ nhost) {
  const int64_t l = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= L) return;
  const int64_t s = starts[l];
  const int64_t e = (l + 1 < L) ? starts[l + 1] - 1 : ((n > 0 && t[n - 1] == '\n') ? n - 1 : n);
  int32_t ty;
  if (e <= s) {
    ty = kEmpty;
  } else if (line_contains(t, s, e, "Time", 4) && line_contains(t, s, e, "XLONG_U", 7)) {
    ty = kHeader;
    atomicMin(first_header, (unsigned long long)l);
  } else {
    bool only = true;
    for (int64_t i = s; i < e; ++i) {
      const char c = t[i];
      if (c != '-' && c != ' ' && c != '\t') {
        only = false;
        break;
      }
    }
    if (only && line_contains(t, s, e, "---", 3)) {
      ty = kSep;
    } else {
      int64_t pos = s;
      int iv[4];
      double dv[4];
      bool ok = true;
      int host = 0;
      for (int f = 0; f < 4 && ok; ++f) ok = extract_int(t, pos, e, iv[f]);
      for (int f = 0; f < 4 && ok; ++f) {
        const int r = extract_double(t, pos, e, dv[f]);
        if (r == 0) ok = false;
        if (r == 2) host = 1;
      }
      ty = !ok ? kBad : (host ? kHost : kData);
      if (ty == kHost) atomicAdd(nhost, 1);
      if (ty == kData) {
        for (int f = 0; f < 4; ++f) {
          ol.ival[l * 4 + f] = iv[f];
          ol.dval[l * 4 + f] = dv[f];
        }
      }
    }
  }
  ol.type[l] = ty;
}

__global__ void obs_sep_kernel(const int32_t* __restrict__ type, int64_t L,
                               const unsigned long long* __restrict__ first_header,
                               unsigned long long* __restrict__ first_sep) {
  const int64_t l = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (l < L && type[l] == kSep && (unsigned long long)l > *first_header) atomicMin(first_sep, (unsigned long long)l);
}

__global__ void obs_keep_kernel(const ObsLines ol, int64_t L, const unsigned long long* __restrict__ first_sep,
                                double missing, int64_t* __restrict__ keep) {
  const int64_t l = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= L) return;
  keep[l] = ((unsigned long long)l > *first_sep && ol.type[l] == kData && ol.dval[l * 4 + 3] != missing) ? 1 : 0;
}

__global__ void obs_write_kernel(const ObsLines ol, int64_t L, const int64_t* __restrict__ keep,
                                 const int64_t* __restrict__ pos, int32_t* __restrict__ xyz,
                                 double* __restrict__ vals) {
  const int64_t l = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= L || !keep[l]) return;
  const int64_t o = pos[l];
  xyz[3 * o + 0] = ol.ival[l * 4 + 3];  // x
  xyz[3 * o + 1] = ol.ival[l * 4 + 2];  // y
  xyz[3 * o + 2] = ol.ival[l * 4 + 1];  // z
  for (int f = 0; f < 4; ++f) vals[4 * o + f] = ol.dval[l * 4 + f];
}

// ---- SimpleState values: per line, doubles until the first failed extraction ----
// Per-line mode after the count pass: 0 = read on the device token-parallel
// (or by the thread-per-line kernels), 1 = read on the host (a number outside
// the fast path), 2 = read on the device by the sequential extraction loop.
enum ValueMode : int32_t { kValFast = 0, kValHost = 1, kValSeq = 2 };

__device__ __forceinline__ void line_span(const char* t, int64_t n, const int64_t* starts, int64_t L, int64_t l,
                                          int64_t& s, int64_t& e) {
  s = starts[l];
  e = (l + 1 < L) ? starts[l + 1] - 1 : ((n > 0 && t[n - 1] == '\n') ? n - 1 : n);
}

// The extraction loop of one line: count, whether a number needs the host,
// and (with out) the values.
__device__ int64_t line_values_seq(const char* t, int64_t s, int64_t e, int& h, double* out) {
  int64_t pos = s, c = 0;
  h = 0;
  double v;
  for (;;) {
    const int r = extract_double(t, pos, e, v);
    if (r == 0) break;
    if (r == 2) h = 1;
    if (out && !h) out[c] = v;
    ++c;
  }
  return c;
}

// Thread per line (short lines).
__global__ void values_count_kernel(const char* __restrict__ t, int64_t n, const int64_t* __restrict__ starts,
                                    int64_t L, int64_t* __restrict__ counts, int32_t* __restrict__ mode,
                                    int32_t* __restrict__ nhost) {
  const int64_t l = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= L) return;
  int64_t s, e;
  line_span(t, n, starts, L, l, s, e);
  int h;
  counts[l] = line_values_seq(t, s, e, h, nullptr);
  mode[l] = h ? kValHost : kValFast;
  if (h) atomicAdd(nhost, 1);
}

__global__ void values_write_kernel(const char* __restrict__ t, int64_t n, const int64_t* __restrict__ starts,
                                    int64_t L, const int64_t* __restrict__ offs, const int32_t* __restrict__ mode,
                                    double* __restrict__ out) {
  const int64_t l = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= L || mode[l] == kValHost) return;
  int64_t s, e;
  line_span(t, n, starts, L, l, s, e);
  int h;
  line_values_seq(t, s, e, h, out + offs[l]);
}

// Warp per line (long lines).  A line whose white-space separated tokens are
// each one number that extract_double consumes whole is "regular": for it
// the extraction sequence is the token sequence (each extraction skips white
// space to the next token start and ends at the token's end; after the last
// token it meets only white space and fails), so the tokens can be read in
// parallel.  Each 512-byte round of the line gives lane i the token starts in
// bytes [16 i, 16 i + 16) as a bit mask, and the lanes then walk their set
// bits together, so that the warp runs one parse per token rank of the round
// instead of one per byte offset at which some lane meets a token; a warp
// prefix sum of the lanes' token counts places the values.  Other lines go
// to the sequential loop (lane 0).
constexpr int kWin = 16;
constexpr int kRound = 32 * kWin;
constexpr int64_t kWarpLineBytes = 256;  // mean line length from which a warp reads each line

// Bit j set: a token (a non-blank byte after a blank or at the line start)
// starts at w0 + j, for w0 + j < w1 <= w0 + kWin.
__device__ __forceinline__ unsigned token_mask(const char* t, int64_t s, int64_t w0, int64_t w1) {
  unsigned m = 0;
  bool prev_ws = w0 == s || (w0 < w1 && is_ws(t[w0 - 1]));
#pragma unroll
  for (int j = 0; j < kWin; ++j) {
    if (w0 + j < w1) {
      const bool ws = is_ws(t[w0 + j]);
      m |= (!ws && prev_ws) ? (1u << j) : 0u;
      prev_ws = ws;
    }
  }
  return m;
}

__global__ void values_count_warp_kernel(const char* __restrict__ t, int64_t n, const int64_t* __restrict__ starts,
                                         int64_t L, int64_t* __restrict__ counts, int32_t* __restrict__ mode,
                                         int32_t* __restrict__ nhost) {
  const int64_t l = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;  // one line per warp
  const int lane = threadIdx.x & 31;
  if (l >= L) return;
  int64_t s, e;
  line_span(t, n, starts, L, l, s, e);
  int c = 0;
  bool bad = false, host = false;
  for (int64_t base = s; base < e; base += kRound) {
    const int64_t w0 = base + (int64_t)lane * kWin;
    const int64_t w1 = w0 + kWin < e ? w0 + kWin : e;
    for (unsigned m = token_mask(t, s, w0, w1); m; m &= m - 1) {
      const int64_t p = w0 + (__ffs(m) - 1);
      int64_t pos = p;
      double v;
      const int r = extract_double(t, pos, e, v);
      if (r != 0 && (pos == e || is_ws(t[pos]))) {
        ++c;
        host |= (r == 2);
      } else {
        bad = true;
      }
    }
  }
  bad = __any_sync(0xffffffffu, bad);
  host = __any_sync(0xffffffffu, host);
  long long cnt = c;  // a line may hold more than 2^31 values
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, off);
  if (lane != 0) return;
  int32_t m;
  if (bad) {
    int h;
    cnt = line_values_seq(t, s, e, h, nullptr);
    m = h ? kValHost : kValSeq;
  } else {
    m = host ? kValHost : kValFast;
  }
  counts[l] = cnt;
  mode[l] = m;
  if (m == kValHost) atomicAdd(nhost, 1);
}

__global__ void values_write_warp_kernel(const char* __restrict__ t, int64_t n, const int64_t* __restrict__ starts,
                                         int64_t L, const int64_t* __restrict__ offs,
                                         const int32_t* __restrict__ mode, double* __restrict__ out) {
  const int64_t l = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (l >= L) return;
  const int32_t m = mode[l];
  if (m == kValHost) return;
  int64_t s, e;
  line_span(t, n, starts, L, l, s, e);
  int64_t o = offs[l];
  if (m == kValSeq) {
    if (lane == 0) {
      int h;
      line_values_seq(t, s, e, h, out + o);
    }
    return;
  }
  for (int64_t base = s; base < e; base += kRound) {
    const int64_t w0 = base + (int64_t)lane * kWin;
    const int64_t w1 = w0 + kWin < e ? w0 + kWin : e;
    const unsigned mask = token_mask(t, s, w0, w1);
    const int cnt = __popc(mask);
    int inc = cnt;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, inc, off);
      if (lane >= off) inc += y;
    }
    int64_t slot = o + inc - cnt;
    for (unsigned m = mask; m; m &= m - 1) {
      int64_t pos = w0 + (__ffs(m) - 1);
      double v;
      extract_double(t, pos, e, v);
      out[slot++] = v;
    }
    o += __shfl_sync(0xffffffffu, inc, 31);
  }
}

// ---- "%12.6f" writer ----
// Exact value of |v| * 10^6 rounded half-to-even, for finite |v| < 2^53.
__device__ bool micro_units(double v, unsigned long long& q) {
  const double a = fabs(v);
  if (!(a < 9007199254740992.0)) return false;
  if (a == 0.0) {
    q = 0;
    return true;
  }
  int e2;
  const double fr = frexp(a, &e2);               // a = fr * 2^e2, fr in [0.5, 1)
  const unsigned long long m = (unsigned long long)ldexp(fr, 53);  // exact 53-bit mantissa
  const int e = e2 - 53;                          // a = m * 2^e
  const unsigned __int128 P = (unsigned __int128)m * 15625u;  // m * 5^6
  const int sh = e + 6;                           // a * 10^6 = P * 2^sh
  if (sh >= 0) {  // sh <= 6 since |v| < 2^53; P << sh < 2^73, so check the high word
    const unsigned __int128 w = P << sh;
    q = (unsigned long long)w;
    return (w >> 64) == 0;
  }
  const int s = -sh;
  if (s >= 100) {
    q = 0;
    return true;
  }
  const unsigned __int128 qq = P >> s;
  const unsigned __int128 rem = P - (qq << s);
  const unsigned __int128 half = (unsigned __int128)1 << (s - 1);
  unsigned __int128 r = qq;
  if (rem > half || (rem == half && (qq & 1))) r += 1;
  if (r >> 64) return false;
  q = (unsigned long long)r;
  return true;
}

// Characters of the formatted value (without padding) into buf; returns the
// length, or -1 if the host must format it.
__device__ int format_f6(double v, char* buf) {
  unsigned long long q;
  if (!micro_units(v, q)) return -1;
  char tmp[40];
  int n = 0;
  unsigned long long ip = q / 1000000ull, fp = q % 1000000ull;
  for (int d = 0; d < 6; ++d) {
    tmp[n++] = (char)('0' + fp % 10);
    fp /= 10;
  }
  tmp[n++] = '.';
  do {
    tmp[n++] = (char)('0' + ip % 10);
    ip /= 10;
  } while (ip);
  if (signbit(v)) tmp[n++] = '-';
  for (int i = 0; i < n; ++i) buf[i] = tmp[n - 1 - i];
  return n;
}

__global__ void fmt_len_kernel(const double* __restrict__ v, int64_t count, int32_t nx, int64_t* __restrict__ len,
                               int32_t* __restrict__ host, int32_t* __restrict__ nhost) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  char buf[40];
  const int n = format_f6(v[i], buf);
  host[i] = n < 0 ? 1 : 0;
  if (n < 0) atomicAdd(nhost, 1);
  const int w = n < 0 ? 0 : (n < 12 ? 12 : n);
  len[i] = w + 1;  // the separator: " " inside a row, "\n" at its end
}

__global__ void fmt_write_kernel(const double* __restrict__ v, int64_t count, int32_t nx,
                                 const int64_t* __restrict__ off, const int32_t* __restrict__ host,
                                 char* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  char* o = out + off[i];
  if (!host[i]) {
    char buf[40];
    const int n = format_f6(v[i], buf);
    const int pad = n < 12 ? 12 - n : 0;
    for (int k = 0; k < pad; ++k) o[k] = ' ';
    for (int k = 0; k < n; ++k) o[pad + k] = buf[k];
    o[pad + n] = ((i + 1) % nx == 0) ? '\n' : ' ';
  }
}

template <typename F>
int with_lines(mg_context* ctx, const char* text, int64_t nbytes, F&& body) {
  cudaStream_t s = ctx->stream;
  const int64_t nch = (nbytes + kChunk - 1) / kChunk;
  mg::Carver cv;
  cv.reserve<char>(nbytes + 1);
  cv.reserve<int64_t>(nch + 1);
  cv.reserve<int64_t>(nch + 1);
  cv.reserve<char>(mg::scan_temp_bytes(nch));
  void* ws = mg::workspace(ctx, cv.off);
  if (!ws) return MG_ERR_NOMEM;
  cv = mg::Carver{static_cast<char*>(ws), 0};
  char* t = cv.take<char>(nbytes + 1);
  int64_t* ccount = cv.take<int64_t>(nch + 1);
  int64_t* coff = cv.take<int64_t>(nch + 1);
  void* tmp = cv.take<char>(mg::scan_temp_bytes(nch));
  MG_TRY_CUDA(cudaMemcpyAsync(t, text, nbytes, cudaMemcpyHostToDevice, s));
  line_count_kernel<<<(unsigned)nch, kThreads, 0, s>>>(t, nbytes, ccount);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(mg::exclusive_scan(ccount, coff, nch, tmp, mg::scan_temp_bytes(nch), s));
  int64_t L = 0;
  MG_TRY_CUDA(cudaMemcpyAsync(&L, coff + nch, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  MG_TRY_CUDA(cudaStreamSynchronize(s));
  // The per-line buffers live in a second allocation: the workspace above
  // holds the text.
  int64_t* starts = nullptr;
  MG_TRY_CUDA(cudaMallocAsync(&starts, sizeof(int64_t) * (L + 1), s));
  line_fill_kernel<<<(unsigned)nch, kThreads, 0, s>>>(t, nbytes, coff, starts);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  const int rc = body(t, L, starts);
  cudaFreeAsync(starts, s);
  return rc;
}

// The lines a host istringstream must read (numbers outside the fast path);
// nflag is the device count of them, so the flags are copied only when some
// are set.
std::vector<int64_t> host_lines(mg_context* ctx, const int32_t* flags, int64_t L, int32_t want, const int32_t* nflag,
                                int* rc) {
  *rc = MG_OK;
  ctx->io_host_items = 0;
  if (L == 0) return {};
  int32_t nf = 0;
  if (cudaMemcpyAsync(&nf, nflag, sizeof(nf), cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
      cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
    *rc = mg::fail(ctx, MG_ERR_CUDA, "text I/O: device copy failed");
    return {};
  }
  if (nf == 0) return {};
  std::vector<int32_t> h(L);
  if (cudaMemcpyAsync(h.data(), flags, sizeof(int32_t) * L, cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
      cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
    *rc = mg::fail(ctx, MG_ERR_CUDA, "text I/O: device copy failed");
    return {};
  }
  std::vector<int64_t> out;
  for (int64_t l = 0; l < L; ++l)
    if (h[l] == want) out.push_back(l);
  ctx->io_host_items = (int64_t)out.size();
  return out;
}

std::string host_line(const char* text, int64_t nbytes, const std::vector<int64_t>& starts, int64_t l) {
  const int64_t s = starts[l];
  int64_t e = (l + 1 < (int64_t)starts.size()) ? starts[l + 1] - 1 : nbytes;
  if (l + 1 >= (int64_t)starts.size() && nbytes > 0 && text[nbytes - 1] == '\n') e = nbytes - 1;
  return std::string(text + s, text + e);
}

}  // namespace

extern "C" {

int mg_parse_grid_obs(mg_context* ctx, const char* text, int64_t nbytes, double missing_value, int32_t* xyz,
                      double* vals, int64_t cap, int64_t* count) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(text && nbytes >= 0 && count, "mg_parse_grid_obs: bad arguments");
  *count = 0;
  if (nbytes == 0) return MG_OK;
  cudaStream_t s = ctx->stream;
  return with_lines(ctx, text, nbytes, [&](const char* t, int64_t L, int64_t* starts) -> int {
    ObsLines ol{};
    unsigned long long* marks = nullptr;  // first header, first separator after it
    int32_t* nhost = nullptr;
    int64_t *keep = nullptr, *pos = nullptr;
    void* tmp = nullptr;
    const size_t tmpb = mg::scan_temp_bytes(L);
    MG_TRY_CUDA(cudaMallocAsync(&ol.type, sizeof(int32_t) * L, s));
    MG_TRY_CUDA(cudaMallocAsync(&ol.ival, sizeof(int32_t) * 4 * L, s));
    MG_TRY_CUDA(cudaMallocAsync(&ol.dval, sizeof(double) * 4 * L, s));
    MG_TRY_CUDA(cudaMallocAsync(&marks, sizeof(unsigned long long) * 2, s));
    MG_TRY_CUDA(cudaMallocAsync(&nhost, sizeof(int32_t), s));
    MG_TRY_CUDA(cudaMallocAsync(&keep, sizeof(int64_t) * (L + 1), s));
    MG_TRY_CUDA(cudaMallocAsync(&pos, sizeof(int64_t) * (L + 1), s));
    MG_TRY_CUDA(cudaMallocAsync(&tmp, tmpb, s));
    auto release = [&]() {
      cudaFreeAsync(ol.type, s);
      cudaFreeAsync(ol.ival, s);
      cudaFreeAsync(ol.dval, s);
      cudaFreeAsync(marks, s);
      cudaFreeAsync(nhost, s);
      cudaFreeAsync(keep, s);
      cudaFreeAsync(pos, s);
      cudaFreeAsync(tmp, s);
    };
    MG_TRY_CUDA(cudaMemsetAsync(marks, 0xff, sizeof(unsigned long long) * 2, s));
    MG_TRY_CUDA(cudaMemsetAsync(nhost, 0, sizeof(int32_t), s));
    const unsigned g = (unsigned)((L + kThreads - 1) / kThreads);
    obs_lines_kernel<<<g, kThreads, 0, s>>>(t, nbytes, starts, L, ol, marks, nhost);
    MG_COUNT_LAUNCH();
    obs_sep_kernel<<<g, kThreads, 0, s>>>(ol.type, L, marks, marks + 1);
    MG_COUNT_LAUNCH();
    MG_TRY_CUDA(cudaGetLastError());
    // Lines with numbers outside the fast path: the reference's own
    // extraction on the host.
    int rc = MG_OK;
    const std::vector<int64_t> hl = host_lines(ctx, ol.type, L, kHost, nhost, &rc);
    if (rc != MG_OK) return release(), rc;
    if (!hl.empty()) {
      std::vector<int64_t> hs(L);
      MG_TRY_CUDA(cudaMemcpyAsync(hs.data(), starts, sizeof(int64_t) * L, cudaMemcpyDeviceToHost, s));
      MG_TRY_CUDA(cudaStreamSynchronize(s));
      for (int64_t l : hl) {
        std::istringstream iss(host_line(text, nbytes, hs, l));
        int time, z, y, x;
        double znu, lon, lat, v;
        int32_t ty = kBad;
        if (iss >> time >> z >> y >> x >> znu >> lon >> lat >> v) {
          const int32_t iv[4] = {time, z, y, x};
          const double dv[4] = {znu, lon, lat, v};
          MG_TRY_CUDA(cudaMemcpyAsync(ol.ival + 4 * l, iv, sizeof(iv), cudaMemcpyHostToDevice, s));
          MG_TRY_CUDA(cudaMemcpyAsync(ol.dval + 4 * l, dv, sizeof(dv), cudaMemcpyHostToDevice, s));
          ty = kData;
        }
        MG_TRY_CUDA(cudaMemcpyAsync(ol.type + l, &ty, sizeof(ty), cudaMemcpyHostToDevice, s));
        MG_TRY_CUDA(cudaStreamSynchronize(s));
      }
    }
    obs_keep_kernel<<<g, kThreads, 0, s>>>(ol, L, marks + 1, missing_value, keep);
    MG_COUNT_LAUNCH();
    MG_TRY_CUDA(mg::exclusive_scan(keep, pos, L, tmp, tmpb, s));
    int64_t total = 0;
    MG_TRY_CUDA(cudaMemcpyAsync(&total, pos + L, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    MG_TRY_CUDA(cudaStreamSynchronize(s));
    *count = total;
    if (total > cap || (total > 0 && (!xyz || !vals))) {
      release();
      return mg::fail(ctx, MG_ERR_CAPACITY, "mg_parse_grid_obs: output arrays too small");
    }
    if (total > 0) {
      obs_write_kernel<<<g, kThreads, 0, s>>>(ol, L, keep, pos, xyz, vals);
      MG_COUNT_LAUNCH();
    }
    MG_TRY_CUDA(cudaGetLastError());
    release();
    return MG_OK;
  });
}

int mg_parse_values(mg_context* ctx, const char* text, int64_t nbytes, double* out, int64_t cap, int64_t* count) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(text && nbytes >= 0 && count, "mg_parse_values: bad arguments");
  *count = 0;
  if (nbytes == 0) return MG_OK;
  cudaStream_t s = ctx->stream;
  return with_lines(ctx, text, nbytes, [&](const char* t, int64_t L, int64_t* starts) -> int {
    int64_t *counts = nullptr, *offs = nullptr;
    int32_t *mode = nullptr, *nhost = nullptr;
    void* tmp = nullptr;
    const size_t tmpb = mg::scan_temp_bytes(L);
    MG_TRY_CUDA(cudaMallocAsync(&counts, sizeof(int64_t) * (L + 1), s));
    MG_TRY_CUDA(cudaMallocAsync(&offs, sizeof(int64_t) * (L + 1), s));
    MG_TRY_CUDA(cudaMallocAsync(&mode, sizeof(int32_t) * L, s));
    MG_TRY_CUDA(cudaMallocAsync(&nhost, sizeof(int32_t), s));
    MG_TRY_CUDA(cudaMallocAsync(&tmp, tmpb, s));
    auto release = [&]() {
      cudaFreeAsync(counts, s);
      cudaFreeAsync(offs, s);
      cudaFreeAsync(mode, s);
      cudaFreeAsync(nhost, s);
      cudaFreeAsync(tmp, s);
    };
    MG_TRY_CUDA(cudaMemsetAsync(nhost, 0, sizeof(int32_t), s));
    // Long lines (a state row per line): a warp per line; short ones: a thread.
    const bool by_warp = nbytes >= kWarpLineBytes * L;
    const unsigned g = (unsigned)((L + kThreads - 1) / kThreads);
    const unsigned gw = (unsigned)((32 * L + kThreads - 1) / kThreads);
    if (by_warp)
      values_count_warp_kernel<<<gw, kThreads, 0, s>>>(t, nbytes, starts, L, counts, mode, nhost);
    else
      values_count_kernel<<<g, kThreads, 0, s>>>(t, nbytes, starts, L, counts, mode, nhost);
    MG_COUNT_LAUNCH();
    MG_TRY_CUDA(cudaGetLastError());
    int rc = MG_OK;
    const std::vector<int64_t> hl = host_lines(ctx, mode, L, kValHost, nhost, &rc);
    if (rc != MG_OK) return release(), rc;
    std::vector<int64_t> hs;
    std::vector<std::vector<double>> hv(hl.size());
    if (!hl.empty()) {
      hs.resize(L);
      MG_TRY_CUDA(cudaMemcpyAsync(hs.data(), starts, sizeof(int64_t) * L, cudaMemcpyDeviceToHost, s));
      MG_TRY_CUDA(cudaStreamSynchronize(s));
      for (size_t q = 0; q < hl.size(); ++q) {
        std::istringstream iss(host_line(text, nbytes, hs, hl[q]));
        double v;
        while (iss >> v) hv[q].push_back(v);
        const int64_t c = (int64_t)hv[q].size();
        MG_TRY_CUDA(cudaMemcpyAsync(counts + hl[q], &c, sizeof(c), cudaMemcpyHostToDevice, s));
        MG_TRY_CUDA(cudaStreamSynchronize(s));
      }
    }
    MG_TRY_CUDA(mg::exclusive_scan(counts, offs, L, tmp, tmpb, s));
    int64_t total = 0;
    MG_TRY_CUDA(cudaMemcpyAsync(&total, offs + L, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    MG_TRY_CUDA(cudaStreamSynchronize(s));
    *count = total;
    if (total > cap || (total > 0 && !out)) {
      release();
      return mg::fail(ctx, MG_ERR_CAPACITY, "mg_parse_values: output array too small");
    }
    if (total > 0) {
      if (by_warp)
        values_write_warp_kernel<<<gw, kThreads, 0, s>>>(t, nbytes, starts, L, offs, mode, out);
      else
        values_write_kernel<<<g, kThreads, 0, s>>>(t, nbytes, starts, L, offs, mode, out);
      MG_COUNT_LAUNCH();
      MG_TRY_CUDA(cudaGetLastError());
      for (size_t q = 0; q < hl.size(); ++q) {
        if (hv[q].empty()) continue;
        int64_t o = 0;
        MG_TRY_CUDA(cudaMemcpyAsync(&o, offs + hl[q], sizeof(o), cudaMemcpyDeviceToHost, s));
        MG_TRY_CUDA(cudaStreamSynchronize(s));
        MG_TRY_CUDA(cudaMemcpyAsync(out + o, hv[q].data(), sizeof(double) * hv[q].size(), cudaMemcpyHostToDevice, s));
      }
      MG_TRY_CUDA(cudaStreamSynchronize(s));
    }
    release();
    return MG_OK;
  });
}

int mg_last_io_host_items(mg_context* ctx, int64_t* count) {
  if (!ctx || !count) return MG_ERR_ARG;
  *count = ctx->io_host_items;
  return MG_OK;
}

int mg_format_state(mg_context* ctx, const double* values, int32_t nx, int32_t ny, char* out, int64_t cap,
                    int64_t* nbytes) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(values && nx > 0 && ny > 0 && nbytes, "mg_format_state: bad arguments");
  cudaStream_t s = ctx->stream;
  const int64_t count = (int64_t)nx * ny;
  const size_t tmpb = mg::scan_temp_bytes(count);
  int64_t *len = nullptr, *off = nullptr;
  int32_t *host = nullptr, *nhost = nullptr;
  void* tmp = nullptr;
  MG_TRY_CUDA(cudaMallocAsync(&len, sizeof(int64_t) * (count + 1), s));
  MG_TRY_CUDA(cudaMallocAsync(&off, sizeof(int64_t) * (count + 1), s));
  MG_TRY_CUDA(cudaMallocAsync(&host, sizeof(int32_t) * count, s));
  MG_TRY_CUDA(cudaMallocAsync(&nhost, sizeof(int32_t), s));
  MG_TRY_CUDA(cudaMallocAsync(&tmp, tmpb, s));
  auto release = [&]() {
    cudaFreeAsync(len, s);
    cudaFreeAsync(off, s);
    cudaFreeAsync(host, s);
    cudaFreeAsync(nhost, s);
    cudaFreeAsync(tmp, s);
  };
  MG_TRY_CUDA(cudaMemsetAsync(nhost, 0, sizeof(int32_t), s));
  const unsigned g = (unsigned)((count + kThreads - 1) / kThreads);
  fmt_len_kernel<<<g, kThreads, 0, s>>>(values, count, nx, len, host, nhost);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  // Values the device does not format: their text length comes from the host.
  int rc = MG_OK;
  const std::vector<int64_t> hl = host_lines(ctx, host, count, 1, nhost, &rc);
  if (rc != MG_OK) return release(), rc;
  std::vector<std::string> htxt(hl.size());
  for (size_t q = 0; q < hl.size(); ++q) {
    double v = 0.0;
    MG_TRY_CUDA(cudaMemcpyAsync(&v, values + hl[q], sizeof(v), cudaMemcpyDeviceToHost, s));
    MG_TRY_CUDA(cudaStreamSynchronize(s));
    std::ostringstream os;
    os << std::fixed;
    os.precision(6);
    os.width(12);
    os << v;
    htxt[q] = os.str() + (((hl[q] + 1) % nx == 0) ? "\n" : " ");
    const int64_t l = (int64_t)htxt[q].size();
    MG_TRY_CUDA(cudaMemcpyAsync(len + hl[q], &l, sizeof(l), cudaMemcpyHostToDevice, s));
    MG_TRY_CUDA(cudaStreamSynchronize(s));
  }
  MG_TRY_CUDA(mg::exclusive_scan(len, off, count, tmp, tmpb, s));
  int64_t total = 0;
  MG_TRY_CUDA(cudaMemcpyAsync(&total, off + count, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  MG_TRY_CUDA(cudaStreamSynchronize(s));
  *nbytes = total;
  if (total > cap || !out) {
    release();
    return out ? mg::fail(ctx, MG_ERR_CAPACITY, "mg_format_state: output buffer too small") : MG_ERR_CAPACITY;
  }
  char* dout = nullptr;
  MG_TRY_CUDA(cudaMallocAsync(&dout, (size_t)total, s));
  fmt_write_kernel<<<g, kThreads, 0, s>>>(values, count, nx, off, host, dout);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  MG_TRY_CUDA(cudaMemcpyAsync(out, dout, (size_t)total, cudaMemcpyDeviceToHost, s));
  MG_TRY_CUDA(cudaStreamSynchronize(s));
  for (size_t q = 0; q < hl.size(); ++q) {
    int64_t o = 0;
    MG_TRY_CUDA(cudaMemcpy(&o, off + hl[q], sizeof(o), cudaMemcpyDeviceToHost));
    std::memcpy(out + o, htxt[q].data(), htxt[q].size());
  }
  cudaFreeAsync(dout, s);
  release();
  return MG_OK;
}

}  // extern "C"
