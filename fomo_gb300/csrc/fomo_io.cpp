// Writers and reader of FoMo cubes (GoftCube::writegoftcube / readgoftcube).
//
// The on-disk formats are the ones FoMo-C writes and its Python reader
// (fomo-c/python/readfomo.py:9-118) consumes:
//   .txt  "FoMo-<version>", dim, ng, nvars, the units tab-separated, the table
//         and abundance file names, then one line per point: the coordinates
//         and variables, 8 significant digits, each followed by a space
//         (fomo-c/src/fomo-io.cpp:26-77);
//   .dat  "FoMo-<version>#", int dim, int ng, int nvars, every unit and the two
//         names as a size_t length + characters, then each coordinate and each
//         variable as ng FP32 values (fomo-io.cpp:89-150);
//   .gz   the gzip of either, written when the zip option is set, optionally
//         deleting the uncompressed file (fomo-io.cpp:154-170, 248-287).
// The gzip stream is this file's own DEFLATE encoder (RFC 1951, below) in an
// RFC 1952 member with a CRC-32 trailer: any gzip reader returns the same
// bytes as the uncompressed file (the compressed bytes differ from the
// reference's Boost/zlib output; their size is about zlib's default level's).
#include <algorithm>
#include <atomic>
#include <charconv>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <iterator>
#include <fstream>
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <system_error>
#include <thread>
#include <vector>

#include "../../include/FoMo.h"

namespace FoMo {
namespace {

const char* const kVersion = "v3.3-gb300";
const char* const kExt[2] = {".dat", ".txt"};

// CRC-32 (IEEE 802.3 polynomial, reflected), as gzip's trailer uses.
struct Crc32Table {
  uint32_t v[256];
  Crc32Table() {
    for (uint32_t i = 0; i < 256; ++i) {
      uint32_t c = i;
      for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
      v[i] = c;
    }
  }
};

uint32_t crc32_update(uint32_t crc, const unsigned char* p, size_t n) {
  static const Crc32Table tab;  // built once, thread-safe (a function-local static)
  const uint32_t* table = tab.v;
  crc = ~crc;
  for (size_t i = 0; i < n; ++i) crc = table[(crc ^ p[i]) & 0xFFu] ^ (crc >> 8);
  return ~crc;
}

void put_le(std::ostream& o, uint32_t v, int bytes) {
  for (int i = 0; i < bytes; ++i) o.put((char)((v >> (8 * i)) & 0xFFu));
}

// ---------------------------------------------------------------------------
// DEFLATE (RFC 1951): greedy LZ77 matching over hash chains in the 32 KB
// window, and Huffman codes made for each chunk's symbols (section 3.2.7), or
// stored blocks where those are smaller.  The data are cut into
// chunks that several threads compress at once; a chunk's matches stay inside
// it, and every chunk but the last ends with an empty stored block (section
// 3.2.4), which brings the bit stream to a byte boundary, so the chunks'
// bytes join as they are.
// ---------------------------------------------------------------------------
class BitWriter {
 public:
  explicit BitWriter(std::vector<unsigned char>& out) : out_(out) {}
  void put(uint32_t bits, int n) {  // n <= 32, least significant bit first
    acc_ |= (uint64_t)bits << nacc_;
    nacc_ += n;
    while (nacc_ >= 8) {
      out_.push_back((unsigned char)(acc_ & 0xFFu));
      acc_ >>= 8;
      nacc_ -= 8;
    }
  }
  void align() {
    if (nacc_ > 0) put(0, 8 - nacc_);
  }

 private:
  std::vector<unsigned char>& out_;
  uint64_t acc_ = 0;
  int nacc_ = 0;
};

// Lengths 3..258 and distances 1..32768: base values and extra bits of their
// codes 257..285 and 0..29 (RFC 1951 section 3.2.5).
const uint16_t kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                               31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,    65,    97,    129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

// Code lengths of a Huffman code for `freq`, none longer than maxbits (RFC
// 1951 codes are at most 15 bits, the code-length code 7): a Huffman tree
// built over the used symbols; while it is too deep, the counts are halved
// (every used symbol stays used) and the tree built again.
std::vector<uint8_t> huffman_lengths(std::vector<uint32_t> freq, int maxbits) {
  std::vector<uint8_t> len(freq.size(), 0);
  for (;;) {
    std::vector<int> syms;
    for (size_t i = 0; i < freq.size(); ++i)
      if (freq[i]) syms.push_back((int)i);
    if (syms.empty()) return len;
    if (syms.size() == 1) {
      len[syms[0]] = 1;
      return len;
    }
    std::vector<uint64_t> w;
    std::vector<int> parent;
    std::vector<std::pair<uint64_t, int>> heap;  // (weight, node), a min-heap
    for (int sym : syms) {
      heap.emplace_back(freq[sym], (int)w.size());
      w.push_back(freq[sym]);
      parent.push_back(-1);
    }
    auto cmp = [](const std::pair<uint64_t, int>& a, const std::pair<uint64_t, int>& b) { return a > b; };
    std::make_heap(heap.begin(), heap.end(), cmp);
    while (heap.size() > 1) {
      std::pop_heap(heap.begin(), heap.end(), cmp);
      const auto a = heap.back();
      heap.pop_back();
      std::pop_heap(heap.begin(), heap.end(), cmp);
      const auto b = heap.back();
      heap.pop_back();
      const int node = (int)w.size();
      w.push_back(a.first + b.first);
      parent.push_back(-1);
      parent[a.second] = parent[b.second] = node;
      heap.emplace_back(a.first + b.first, node);
      std::push_heap(heap.begin(), heap.end(), cmp);
    }
    int deepest = 0;
    for (size_t k = 0; k < syms.size(); ++k) {
      int depth = 0;
      for (int v = (int)k; parent[v] >= 0; v = parent[v]) ++depth;
      len[syms[k]] = (uint8_t)depth;
      deepest = std::max(deepest, depth);
    }
    if (deepest <= maxbits) return len;
    for (uint32_t& f : freq)
      if (f) f = (f + 1) / 2;
    std::fill(len.begin(), len.end(), 0);
  }
}

// Canonical codes of the lengths (RFC 1951 section 3.2.2), bit-reversed for
// the least-significant-bit-first writer.
std::vector<uint16_t> canonical_codes(const std::vector<uint8_t>& len) {
  int count[16] = {0}, next[16] = {0};
  for (uint8_t l : len)
    if (l) ++count[l];
  for (int bits = 1, code = 0; bits < 16; ++bits) {
    code = (code + count[bits - 1]) << 1;
    next[bits] = code;
  }
  std::vector<uint16_t> out(len.size(), 0);
  for (size_t s = 0; s < len.size(); ++s) {
    if (!len[s]) continue;
    uint32_t c = (uint32_t)next[len[s]]++, r = 0;
    for (int i = 0; i < len[s]; ++i, c >>= 1) r = (r << 1) | (c & 1u);
    out[s] = (uint16_t)r;
  }
  return out;
}

int dist_code(uint32_t d) {  // 1 <= d <= 32768
  if (d <= 4) return (int)d - 1;
  const uint32_t d1 = d - 1;
  int nb = 31;
  while (!(d1 >> nb)) --nb;  // the top bit of d1 (>= 2)
  return 2 * nb + (int)((d1 >> (nb - 1)) & 1u);
}

int len_code(int l) {  // 3 <= l <= 258: code - 257
  int c = 0;
  while (c < 28 && kLenBase[c + 1] <= l) ++c;
  return c;
}

// One chunk: LZ77 tokens, then one block with Huffman codes made for them
// (BTYPE 10), or stored blocks when those are smaller (incompressible data).
void deflate_chunk(const unsigned char* d, size_t n, bool final, std::vector<unsigned char>& out) {
  constexpr int kHashBits = 15, kWindow = 32768, kMaxChain = 32, kMaxLen = 258;
  // tokens: dist == 0: the literal `lit`; else a match of length `lit`
  struct Tok {
    uint16_t lit, dist;
  };
  std::vector<Tok> toks;
  toks.reserve(n / 3 + 16);
  std::vector<int32_t> head(size_t(1) << kHashBits, -1), prev(kWindow, -1);
  auto hash = [&](size_t i) {
    return (((uint32_t)d[i] << 10) ^ ((uint32_t)d[i + 1] << 5) ^ (uint32_t)d[i + 2]) & ((1u << kHashBits) - 1u);
  };
  auto insert = [&](size_t i) {
    if (i + 2 >= n) return;
    const uint32_t h = hash(i);
    prev[i & (kWindow - 1)] = head[h];
    head[h] = (int32_t)i;
  };
  std::vector<uint32_t> lf(286, 0), df(30, 0);
  for (size_t i = 0; i < n;) {
    int best_len = 0;
    size_t best_dist = 0;
    if (i + 2 < n) {
      const int maxlen = (int)std::min<size_t>(kMaxLen, n - i);
      int32_t j = head[hash(i)];
      for (int chain = 0; j >= 0 && i - (size_t)j <= (size_t)kWindow && chain < kMaxChain; ++chain) {
        if (d[j + best_len] == d[i + best_len]) {
          int l = 0;
          while (l < maxlen && d[j + l] == d[i + l]) ++l;
          if (l > best_len) {
            best_len = l;
            best_dist = i - (size_t)j;
            if (l == maxlen) break;
          }
        }
        const int32_t nj = prev[j & (kWindow - 1)];
        if (nj >= j) break;  // the ring slot was reused by a later position
        j = nj;
      }
    }
    if (best_len >= 3) {
      toks.push_back({(uint16_t)best_len, (uint16_t)best_dist});
      ++lf[257 + len_code(best_len)];
      ++df[dist_code((uint32_t)best_dist)];
      for (int k = 0; k < best_len; ++k) insert(i + (size_t)k);
      i += (size_t)best_len;
    } else {
      toks.push_back({d[i], 0});
      ++lf[d[i]];
      insert(i);
      ++i;
    }
  }
  lf[256] = 1;  // end of block
  int used = 0;
  for (uint32_t f : lf) used += f ? 1 : 0;
  if (used < 2) lf[0] = std::max<uint32_t>(lf[0], 1);  // two codes at least in each tree
  used = 0;
  for (uint32_t f : df) used += f ? 1 : 0;
  if (used < 2) df[0] = std::max<uint32_t>(df[0], 1), df[1] = std::max<uint32_t>(df[1], 1);
  const std::vector<uint8_t> ll = huffman_lengths(lf, 15), dl = huffman_lengths(df, 15);
  const std::vector<uint16_t> lcode = canonical_codes(ll), dcode = canonical_codes(dl);
  int hlit = 286, hdist = 30;
  while (hlit > 257 && !ll[hlit - 1]) --hlit;
  while (hdist > 1 && !dl[hdist - 1]) --hdist;
  // the code lengths, run-length coded with symbols 0-18 (section 3.2.7)
  std::vector<uint8_t> seq(ll.begin(), ll.begin() + hlit);
  seq.insert(seq.end(), dl.begin(), dl.begin() + hdist);
  std::vector<std::pair<uint8_t, uint8_t>> rle;  // (symbol, extra value)
  for (size_t i = 0; i < seq.size();) {
    size_t r = 1;
    while (i + r < seq.size() && seq[i + r] == seq[i]) ++r;
    if (seq[i] == 0 && r >= 3) {
      const size_t k = std::min<size_t>(r, 138);
      rle.emplace_back(k >= 11 ? 18 : 17, (uint8_t)(k >= 11 ? k - 11 : k - 3));
      i += k;
    } else if (seq[i] != 0 && r >= 4) {
      rle.emplace_back(seq[i], 0);
      const size_t k = std::min<size_t>(r - 1, 6);
      rle.emplace_back(16, (uint8_t)(k - 3));
      i += 1 + k;
    } else {
      rle.emplace_back(seq[i], 0);
      ++i;
    }
  }
  std::vector<uint32_t> cf(19, 0);
  for (const auto& e : rle) ++cf[e.first];
  const std::vector<uint8_t> cl = huffman_lengths(cf, 7);
  const std::vector<uint16_t> ccode = canonical_codes(cl);
  static const int kOrder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
  int hclen = 19;
  while (hclen > 4 && !cl[kOrder[hclen - 1]]) --hclen;
  // the block's size, against stored blocks of the same bytes
  uint64_t bits = 3 + 14 + 3 * (uint64_t)hclen;
  for (const auto& e : rle) bits += cl[e.first] + (e.first == 16 ? 2 : e.first == 17 ? 3 : e.first == 18 ? 7 : 0);
  for (const Tok& t : toks) {
    if (!t.dist) {
      bits += ll[t.lit];
    } else {
      const int lc = len_code(t.lit), dc = dist_code(t.dist);
      bits += ll[257 + lc] + kLenExtra[lc] + dl[dc] + kDistExtra[dc];
    }
  }
  bits += ll[256] + (final ? 0 : 3 + 7 + 32);
  const uint64_t stored = (uint64_t)n + 5 * std::max<uint64_t>(1, (n + 65534) / 65535);
  if (bits / 8 + 1 >= stored) {
    // stored blocks (the chunk starts on a byte boundary, and so ends)
    size_t pos = 0;
    do {
      const size_t len = std::min<size_t>(65535, n - pos);
      const bool last = final && pos + len == n;
      out.push_back((unsigned char)(last ? 1 : 0));  // BFINAL, BTYPE 00, padded to the byte
      out.push_back((unsigned char)(len & 0xFFu));
      out.push_back((unsigned char)(len >> 8));
      out.push_back((unsigned char)(~len & 0xFFu));
      out.push_back((unsigned char)((~len >> 8) & 0xFFu));
      out.insert(out.end(), d + pos, d + pos + len);
      pos += len;
    } while (pos < n);
    return;
  }
  BitWriter w(out);
  w.put(final ? 1u : 0u, 1);
  w.put(2u, 2);  // BTYPE 10: codes of this block
  w.put((uint32_t)(hlit - 257), 5);
  w.put((uint32_t)(hdist - 1), 5);
  w.put((uint32_t)(hclen - 4), 4);
  for (int k = 0; k < hclen; ++k) w.put(cl[kOrder[k]], 3);
  for (const auto& e : rle) {
    w.put(ccode[e.first], cl[e.first]);
    if (e.first == 16) w.put(e.second, 2);
    else if (e.first == 17) w.put(e.second, 3);
    else if (e.first == 18) w.put(e.second, 7);
  }
  for (const Tok& t : toks) {
    if (!t.dist) {
      w.put(lcode[t.lit], ll[t.lit]);
      continue;
    }
    const int lc = len_code(t.lit), dc = dist_code(t.dist);
    w.put(lcode[257 + lc], ll[257 + lc]);
    if (kLenExtra[lc]) w.put((uint32_t)(t.lit - kLenBase[lc]), kLenExtra[lc]);
    w.put(dcode[dc], dl[dc]);
    if (kDistExtra[dc]) w.put((uint32_t)(t.dist - kDistBase[dc]), kDistExtra[dc]);
  }
  w.put(lcode[256], ll[256]);  // end of block
  if (!final) {
    w.put(0u, 3);  // an empty stored block, not final: aligns to the byte
    w.align();
    out.push_back(0x00);
    out.push_back(0x00);
    out.push_back(0xFF);
    out.push_back(0xFF);
  } else {
    w.align();
  }
}

// src -> dst as one gzip member (RFC 1952) of the deflated bytes.
bool gzip_file(const std::string& src, const std::string& dst) {
  std::ifstream in(src, std::ios::binary);
  if (!in) return false;
  std::vector<unsigned char> data((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
  constexpr size_t kChunk = size_t(1) << 20;
  const size_t nchunks = std::max<size_t>(1, (data.size() + kChunk - 1) / kChunk);
  std::vector<std::vector<unsigned char>> packed(nchunks);
  std::atomic<size_t> next{0};
  auto work = [&]() {
    for (size_t c; (c = next.fetch_add(1)) < nchunks;) {
      const size_t b = c * kChunk, e = std::min(data.size(), b + kChunk);
      packed[c].reserve((e - b) / 2 + 64);
      deflate_chunk(data.data() + b, e - b, c + 1 == nchunks, packed[c]);
    }
  };
  const unsigned nthreads = std::max(1u, std::min({std::thread::hardware_concurrency(), 16u, (unsigned)nchunks}));
  std::vector<std::thread> pool;
  try {
    for (unsigned t = 1; t < nthreads; ++t) pool.emplace_back(work);
  } catch (const std::system_error&) {
    // no thread to be had: this one compresses the chunks left
  }
  const uint32_t crc = crc32_update(0, data.data(), data.size());  // beside the compressing threads
  work();
  for (std::thread& th : pool) th.join();
  std::ofstream out(dst, std::ios::binary);
  if (!out) return false;
  // header: magic, deflate, no flags, no mtime, no extra flags, OS unknown
  const unsigned char hdr[10] = {0x1f, 0x8b, 8, 0, 0, 0, 0, 0, 0, 255};
  out.write(reinterpret_cast<const char*>(hdr), sizeof(hdr));
  for (const std::vector<unsigned char>& p : packed) out.write(reinterpret_cast<const char*>(p.data()), (std::streamsize)p.size());
  put_le(out, crc, 4);
  put_le(out, (uint32_t)(data.size() & 0xFFFFFFFFu), 4);
  return (bool)out;
}

}  // namespace

// One value of the text format's body as the reference's stream writes it at
// precision 8: the float widened to double, in printf's "%.8g" form in the
// "C" locale (which std::to_chars with chars_format::general and a precision
// reproduces exactly), then a space.  At most 15 characters plus the space.
static char* put_text_value(char* p, char* end, float v) {
  const std::to_chars_result r = std::to_chars(p, end, (double)v, std::chars_format::general, 8);
  *r.ptr = ' ';
  return r.ptr + 1;
}

// The text format (fomo-io.cpp:26-77).  Its body is one line per point, the
// reference writes it through the stream one value at a time and flushes
// every line; here blocks of lines are formatted by several threads at once
// into memory and written in order, with the same bytes.
static void write_text(GoftCube& c, const std::string& filename) {
  std::ofstream out(filename, std::ios::ate | std::ios::binary);
  if (!out.is_open()) {
    std::cerr << "Unable to write to " << filename << std::endl;
    return;
  }
  const int nvars = c.readnvars(), dim = c.readdim(), ng = c.readngrid();
  out << "FoMo-" << kVersion << '\n';
  out << dim << '\n' << ng << '\n' << nvars << '\n';
  const std::vector<std::string> units = c.readunit();
  for (int u = 0; u < dim + nvars; ++u) out << units.at(u) << "\t";
  out << '\n';
  out << c.readchiantifile() << '\n';
  out << c.readabundfile() << '\n';
  const tgrid grid = c.readgrid();
  tvars vars;
  for (int i = 0; i < nvars; ++i) vars.push_back(c.readvar(i));
  std::vector<const float*> cols;
  for (int i = 0; i < dim; ++i) cols.push_back(grid[i].data());
  for (int i = 0; i < nvars; ++i) cols.push_back(vars[i].data());
  const size_t ncol = cols.size();
  const size_t line_max = 16 * ncol + 1;
  constexpr int kLinesPerBlock = 1 << 15;
  const int nblocks = (ng + kLinesPerBlock - 1) / kLinesPerBlock;
  const int nthreads =
      (int)std::max(1u, std::min({std::thread::hardware_concurrency(), 16u, (unsigned)std::max(nblocks, 1)}));
  std::vector<std::vector<char>> buf(nthreads, std::vector<char>(line_max * kLinesPerBlock));
  std::vector<size_t> used(nthreads, 0);
  auto format = [&](int t, int blk) {
    char* const b = buf[t].data();
    char* p = b;
    char* const end = b + buf[t].size();
    const int64_t j1 = std::min<int64_t>(ng, (int64_t)(blk + 1) * kLinesPerBlock);
    for (int64_t j = (int64_t)blk * kLinesPerBlock; j < j1; ++j) {
      for (size_t i = 0; i < ncol; ++i) p = put_text_value(p, end, cols[i][j]);
      *p++ = '\n';
    }
    used[t] = (size_t)(p - b);
  };
  // waves of nthreads blocks: formatted in parallel, written in block order
  for (int b0 = 0; b0 < nblocks; b0 += nthreads) {
    const int nb = std::min(nthreads, nblocks - b0);
    std::vector<std::thread> pool;
    int t = 1;
    try {
      for (; t < nb; ++t) pool.emplace_back(format, t, b0 + t);
    } catch (const std::system_error&) {
      // no thread to be had: this one formats the blocks left
    }
    for (int u = t; u < nb; ++u) format(u, b0 + u);
    format(0, b0);
    for (std::thread& th : pool) th.join();
    for (int k = 0; k < nb; ++k) out.write(buf[k].data(), (std::streamsize)used[k]);
  }
}

static void write_binary(GoftCube& c, const std::string& filename) {
  std::ofstream out(filename, std::ios::binary | std::ios::ate);
  if (!out.is_open()) {
    std::cerr << "Unable to write to " << filename << std::endl;
    return;
  }
  const std::string version = std::string("FoMo-") + kVersion + "#";  // '#' ends the version for readers
  out.write(version.data(), (std::streamsize)version.size());
  const int nvars = c.readnvars(), dim = c.readdim(), ng = c.readngrid();
  out.write(reinterpret_cast<const char*>(&dim), sizeof(dim));
  out.write(reinterpret_cast<const char*>(&ng), sizeof(ng));
  out.write(reinterpret_cast<const char*>(&nvars), sizeof(nvars));
  auto put_string = [&](const std::string& s) {
    const size_t n = s.size();
    out.write(reinterpret_cast<const char*>(&n), sizeof(n));
    out.write(s.data(), (std::streamsize)n);
  };
  const std::vector<std::string> units = c.readunit();
  for (int i = 0; i < dim + nvars; ++i) put_string(units.at(i));
  put_string(c.readchiantifile());
  put_string(c.readabundfile());
  const tgrid grid = c.readgrid();
  for (int i = 0; i < dim; ++i)
    out.write(reinterpret_cast<const char*>(grid[i].data()), (std::streamsize)(sizeof(float) * (size_t)ng));
  for (int i = 0; i < nvars; ++i) {
    const tphysvar v = c.readvar(i);
    out.write(reinterpret_cast<const char*>(v.data()), (std::streamsize)(sizeof(float) * (size_t)ng));
  }
}

// filename's extension is replaced by .dat / .txt (and .gz appended) as the
// options ask (fomo-io.cpp:248-287).
void GoftCube::writegoftcube(const std::string filename) {
  const size_t dot = filename.rfind('.');
  const std::string root = (dot == std::string::npos || dot == 0) ? filename : filename.substr(0, dot);
  if (writeoptions[0]) write_binary(*this, root + kExt[0]);
  if (writeoptions[1]) write_text(*this, root + kExt[1]);
  if (writeoptions[2] && (writeoptions[0] || writeoptions[1])) {
    for (int i = 0; i < 2; ++i) {
      if (!writeoptions[i]) continue;
      const std::string f = root + kExt[i];
      if (!gzip_file(f, f + ".gz")) std::cerr << "Unable to write to " << f << ".gz" << std::endl;
    }
    if (writeoptions[3])
      for (int i = 0; i < 2; ++i)
        if (writeoptions[i]) std::remove((root + kExt[i]).c_str());
  } else if (writeoptions[2]) {
    std::cerr << "Zipping of output only possible if output set with goftcube.setwriteouttext or "
                 "goftcube.setwriteoutbinary."
              << std::endl;
  }
}

// The values of a text cube's body: `count` whitespace-separated numbers, value
// t into cols[t % ncol][t / ncol].  The stream reads each with strtof in the
// "C" locale (correctly rounded); std::from_chars is correctly rounded too, so
// a token it takes whole, as a finite float, gives the stream's value.  The
// tokens are parsed by several threads, each on a stretch of whole tokens.
// False when any token is not of that plain form (a sign '+', a value out of
// the float range, text): the caller then reads the body through the stream,
// with the stream's own rules for such tokens.
static bool parse_text_values(const std::string& body, size_t count, const std::vector<float*>& cols) {
  const size_t ncol = cols.size();
  const char* const b = body.data();
  const size_t len = body.size();
  auto space = [](char c) { return c == ' ' || c == '\n' || c == '\t' || c == '\r' || c == '\v' || c == '\f'; };
  const int nthreads = (int)std::max(
      1u, std::min({std::thread::hardware_concurrency(), 16u, (unsigned)std::max<size_t>(1, len >> 20)}));
  // stretch k: [cut[k], cut[k+1]), cut at the end of the token the even split falls in
  std::vector<size_t> cut(nthreads + 1, len);
  cut[0] = 0;
  for (int k = 1; k < nthreads; ++k) {
    size_t p = std::max(cut[k - 1], len / nthreads * k);
    while (p < len && !space(b[p])) ++p;
    cut[k] = p;
  }
  std::vector<size_t> ntok(nthreads, 0);
  std::vector<char> ok(nthreads, 1);
  auto run = [&](auto&& fn) {
    std::vector<std::thread> pool;
    int t = 1;
    try {
      for (; t < nthreads; ++t) pool.emplace_back(fn, t);
    } catch (const std::system_error&) {
      // no thread to be had: this one takes the stretches left
    }
    for (int u = t; u < nthreads; ++u) fn(u);
    fn(0);
    for (std::thread& th : pool) th.join();
  };
  // pass 1: tokens per stretch
  run([&](int k) {
    size_t n = 0;
    for (size_t p = cut[k]; p < cut[k + 1];) {
      while (p < cut[k + 1] && space(b[p])) ++p;
      if (p == cut[k + 1]) break;
      ++n;
      while (p < cut[k + 1] && !space(b[p])) ++p;
    }
    ntok[k] = n;
  });
  std::vector<size_t> first(nthreads, 0);
  for (int k = 1; k < nthreads; ++k) first[k] = first[k - 1] + ntok[k - 1];
  if (first[nthreads - 1] + ntok[nthreads - 1] < count) return false;  // too few values: the stream's error
  // pass 2: the values, as far as `count`
  run([&](int k) {
    size_t t = first[k];
    for (size_t p = cut[k]; p < cut[k + 1] && t < count;) {
      while (p < cut[k + 1] && space(b[p])) ++p;
      if (p == cut[k + 1]) break;
      size_t q = p;
      while (q < cut[k + 1] && !space(b[q])) ++q;
      float v = 0.0f;
      const std::from_chars_result r = std::from_chars(b + p, b + q, v, std::chars_format::general);
      if (r.ec != std::errc() || r.ptr != b + q || !std::isfinite(v)) {
        ok[k] = 0;
        return;
      }
      cols[t % ncol][t / ncol] = v;
      ++t;
      p = q;
    }
  });
  return std::all_of(ok.begin(), ok.end(), [](char c) { return c != 0; });
}

// Reads a cube written by writegoftcube: the binary (.dat) or text (.txt)
// format above, or the header-less text format of FoMo before 3.4 (dim, ng,
// nvars, table, abundance file, then the values).  lambda0 is taken from the
// table file when it can be read.
void GoftCube::readgoftcube(const std::string emissionsave) {
  std::ifstream in(emissionsave, std::ios::binary);
  if (!in.is_open()) {
    std::cerr << "Unable to read " << emissionsave << std::endl;
    return;
  }
  char first[5] = {0};
  in.read(first, 5);
  const bool versioned = in.gcount() == 5 && std::string(first, 5) == "FoMo-";
  std::string line;
  int rdim = 0, rng = 0, rnvars = 0;
  std::vector<std::string> runits;
  tgrid rgrid;
  tvars rvars;
  // a binary file has its version terminated by '#' on the first line
  bool binary = false;
  if (versioned) {
    std::string rest;
    char ch = 0;
    while (in.get(ch) && ch != '\n' && ch != '#') rest.push_back(ch);
    binary = ch == '#';
  } else {
    in.seekg(0);
  }
  if (binary) {
    in.read(reinterpret_cast<char*>(&rdim), sizeof(rdim));
    in.read(reinterpret_cast<char*>(&rng), sizeof(rng));
    in.read(reinterpret_cast<char*>(&rnvars), sizeof(rnvars));
    if (!in || rdim < 1 || rng < 0 || rnvars < 0) throw std::runtime_error("FoMo: malformed cube file " + emissionsave);
    auto get_string = [&]() {
      size_t n = 0;
      in.read(reinterpret_cast<char*>(&n), sizeof(n));
      if (!in || n > (1u << 20)) throw std::runtime_error("FoMo: malformed cube file " + emissionsave);
      std::string s(n, '\0');
      in.read(&s[0], (std::streamsize)n);
      return s;
    };
    for (int i = 0; i < rdim + rnvars; ++i) runits.push_back(get_string());
    chiantifile = get_string();
    abundfile = get_string();
    rgrid.assign(rdim, tcoord(rng));
    rvars.assign(rnvars, tphysvar(rng));
    for (int i = 0; i < rdim; ++i) in.read(reinterpret_cast<char*>(rgrid[i].data()), sizeof(float) * (size_t)rng);
    for (int i = 0; i < rnvars; ++i) in.read(reinterpret_cast<char*>(rvars[i].data()), sizeof(float) * (size_t)rng);
    if (!in) throw std::runtime_error("FoMo: truncated cube file " + emissionsave);
  } else {
    in >> rdim >> rng >> rnvars;
    if (!in || rdim < 1 || rng < 0 || rnvars < 0) throw std::runtime_error("FoMo: malformed cube file " + emissionsave);
    std::getline(in, line);  // end of the nvars line
    if (versioned) {
      std::getline(in, line);  // units, tab-separated
      std::istringstream us(line);
      std::string u;
      while (std::getline(us, u, '\t')) runits.push_back(u);
      runits.resize(rdim + rnvars);
      std::getline(in, chiantifile);
      std::getline(in, abundfile);
    } else {
      in >> chiantifile >> abundfile;
      runits.assign(rdim + rnvars, "");
    }
    rgrid.assign(rdim, tcoord(rng));
    rvars.assign(rnvars, tphysvar(rng));
    std::vector<float*> cols;
    for (int i = 0; i < rdim; ++i) cols.push_back(rgrid[i].data());
    for (int i = 0; i < rnvars; ++i) cols.push_back(rvars[i].data());
    // the rest of the file, in one read
    const std::streampos here = in.tellg();
    in.seekg(0, std::ios::end);
    const std::streamoff rest = in.tellg() - here;
    in.seekg(here);
    std::string body((size_t)std::max<std::streamoff>(rest, 0), '\0');
    in.read(&body[0], (std::streamsize)body.size());
    body.resize((size_t)in.gcount());
    if (!parse_text_values(body, (size_t)rng * cols.size(), cols)) {
      // value by value through the stream, as the reference reads them
      std::istringstream bs(body);
      for (int j = 0; j < rng; ++j) {
        for (int i = 0; i < rdim; ++i) bs >> rgrid[i][j];
        for (int i = 0; i < rnvars; ++i) bs >> rvars[i][j];
      }
      if (!bs) throw std::runtime_error("FoMo: truncated cube file " + emissionsave);
    }
  }
  dim = (unsigned int)rdim;
  ng = (unsigned int)rng;
  nvars = (unsigned int)rnvars;
  grid = std::move(rgrid);
  vars = std::move(rvars);
  unit = std::move(runits);
  std::ifstream t(chiantifile);
  std::string ion;
  double l0;
  if (t >> ion >> l0) lambda0 = l0;
}

}  // namespace FoMo
