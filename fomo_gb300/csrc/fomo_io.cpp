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
// The gzip stream is made of stored (uncompressed) deflate blocks (RFC 1951
// section 3.2.4) in an RFC 1952 member with a CRC-32 trailer: any gzip reader
// returns the same bytes as the uncompressed file.
#include <algorithm>
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

// src -> dst as one gzip member of stored deflate blocks.
bool gzip_file(const std::string& src, const std::string& dst) {
  std::ifstream in(src, std::ios::binary);
  if (!in) return false;
  std::vector<unsigned char> data((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
  std::ofstream out(dst, std::ios::binary);
  if (!out) return false;
  // header: magic, deflate, no flags, no mtime, no extra flags, OS unknown
  const unsigned char hdr[10] = {0x1f, 0x8b, 8, 0, 0, 0, 0, 0, 0, 255};
  out.write(reinterpret_cast<const char*>(hdr), sizeof(hdr));
  size_t pos = 0;
  do {
    const size_t len = std::min<size_t>(65535, data.size() - pos);
    const bool last = pos + len == data.size();
    out.put((char)(last ? 1 : 0));  // BFINAL, BTYPE = 00 (stored), padded to the byte
    put_le(out, (uint32_t)len, 2);
    put_le(out, (uint32_t)(~len & 0xFFFFu), 2);
    out.write(reinterpret_cast<const char*>(data.data() + pos), (std::streamsize)len);
    pos += len;
  } while (pos < data.size());
  put_le(out, crc32_update(0, data.data(), data.size()), 4);
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
