// NumPy .npz archives of FP64 arrays (host code): the container of the wavefunction restart
// files (reference src/tblite/wavefunction/restart.f90 through src/tblite/io/numpy: a zip
// archive of stored, uncompressed .npy members, CRC-32 checked).
//
// Writing: one stored zip member "<name>.npy" per array, an .npy version 1.0 header
// ({'descr': '<f8', 'fortran_order': True, 'shape': (...), }) padded to a multiple of 64 bytes,
// the data in Fortran order; local headers, central directory and end record as in the zip
// application note (no data descriptors, no zip64, so members stay below 4 GiB).
// Reading: the end record locates the central directory; members must be stored (method 0),
// their CRC-32 is checked; .npy version 1.0 and 2.0 headers with descr '<f8' are accepted, C-order
// arrays are transposed into Fortran order.
#include "npz.h"

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <stdexcept>

namespace tb {

namespace {

uint32_t crc32_of(const unsigned char* p, size_t n) {
  static uint32_t table[256];
  static bool ready = false;
  if (!ready) {  // reflected polynomial 0xEDB88320 (IEEE 802.3)
    for (uint32_t i = 0; i < 256; ++i) {
      uint32_t c = i;
      for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
      table[i] = c;
    }
    ready = true;
  }
  uint32_t c = 0xFFFFFFFFu;
  for (size_t i = 0; i < n; ++i) c = table[(c ^ p[i]) & 0xFFu] ^ (c >> 8);
  return c ^ 0xFFFFFFFFu;
}

void put16(std::vector<unsigned char>& b, uint32_t v) {
  b.push_back((unsigned char)(v & 0xFF));
  b.push_back((unsigned char)((v >> 8) & 0xFF));
}
void put32(std::vector<unsigned char>& b, uint32_t v) {
  put16(b, v & 0xFFFF);
  put16(b, v >> 16);
}
uint32_t get16(const unsigned char* p) { return (uint32_t)p[0] | ((uint32_t)p[1] << 8); }
uint32_t get32(const unsigned char* p) { return get16(p) | (get16(p + 2) << 16); }

std::vector<unsigned char> npy_bytes(const NpyArray& a) {
  std::string shape = "(";  // "(3, 4)", "(5,)" for one axis
  for (size_t i = 0; i < a.shape.size(); ++i) {
    if (i) shape += ", ";
    shape += std::to_string(a.shape[i]);
  }
  if (a.shape.size() == 1) shape += ",";
  shape += ")";
  std::string hdr = "{'descr': '<f8', 'fortran_order': True, 'shape': " + shape + ", }";
  const size_t total = 10 + hdr.size() + 1;
  hdr.append((64 - total % 64) % 64, ' ');
  hdr += '\n';
  std::vector<unsigned char> out;
  const unsigned char magic[6] = {0x93, 'N', 'U', 'M', 'P', 'Y'};
  out.insert(out.end(), magic, magic + 6);
  out.push_back(1);
  out.push_back(0);
  put16(out, (uint32_t)hdr.size());
  out.insert(out.end(), hdr.begin(), hdr.end());
  const unsigned char* d = reinterpret_cast<const unsigned char*>(a.data.data());
  out.insert(out.end(), d, d + a.data.size() * sizeof(double));  // little-endian hosts
  return out;
}

NpyArray npy_parse(const unsigned char* p, size_t n, const std::string& name) {
  auto bad = [&](const char* why) {
    throw std::runtime_error("npz member '" + name + "': " + why);
  };
  if (n < 10 || p[0] != 0x93 || std::memcmp(p + 1, "NUMPY", 5) != 0) bad("not an .npy array");
  size_t hlen = 0, off = 0;
  if (p[6] == 1) {
    hlen = get16(p + 8);
    off = 10;
  } else if (p[6] == 2 || p[6] == 3) {
    if (n < 12) bad("truncated header");
    hlen = get32(p + 8);
    off = 12;
  } else {
    bad("unsupported .npy version");
  }
  if (off + hlen > n) bad("truncated header");
  const std::string hdr(reinterpret_cast<const char*>(p + off), hlen);
  if (hdr.find("'<f8'") == std::string::npos) bad("only little-endian float64 arrays are read");
  const bool fortran = hdr.find("'fortran_order': True") != std::string::npos;
  const size_t sp = hdr.find("'shape':");
  if (sp == std::string::npos) bad("no shape");
  const size_t lp = hdr.find('(', sp), rp = hdr.find(')', sp);
  if (lp == std::string::npos || rp == std::string::npos) bad("bad shape");
  NpyArray a;
  // every element must fit in the member: count stays <= n / 8, so the products below cannot
  // overflow (each factor is checked against that bound before multiplying)
  const size_t max_count = n / sizeof(double);
  size_t count = 1;
  for (size_t i = lp + 1; i < rp;) {
    while (i < rp && (hdr[i] == ' ' || hdr[i] == ',')) ++i;
    if (i >= rp) break;
    if (hdr[i] < '0' || hdr[i] > '9') bad("bad shape");
    size_t v = 0;
    while (i < rp && hdr[i] >= '0' && hdr[i] <= '9') {
      v = 10 * v + (size_t)(hdr[i++] - '0');
      if (v > max_count) bad("truncated data");
    }
    if (i < rp && hdr[i] != ' ' && hdr[i] != ',') bad("bad shape");
    a.shape.push_back(v);
    if (v != 0 && count > max_count / v) bad("truncated data");
    count *= v;
  }
  const size_t data = off + hlen;
  if (data > n || count > (n - data) / sizeof(double)) bad("truncated data");
  std::vector<double> raw(count);
  std::memcpy(raw.data(), p + data, count * sizeof(double));
  if (fortran || a.shape.size() < 2) {
    a.data = std::move(raw);
  } else {  // C order -> Fortran order
    a.data.resize(count);
    const size_t nd = a.shape.size();
    std::vector<size_t> idx(nd, 0);
    for (size_t c = 0; c < count; ++c) {  // c walks C order (last index fastest)
      size_t f = 0, stride = 1;
      for (size_t k = 0; k < nd; ++k) {
        f += idx[k] * stride;
        stride *= a.shape[k];
      }
      a.data[f] = raw[c];
      for (size_t k = nd; k-- > 0;) {
        if (++idx[k] < a.shape[k]) break;
        idx[k] = 0;
      }
    }
  }
  return a;
}

}  // namespace

void npz_write(const std::string& file, const std::vector<std::pair<std::string, NpyArray>>& arrays) {
  std::vector<unsigned char> zip, central;
  uint32_t count = 0;
  for (const auto& [name, arr] : arrays) {
    const std::string member = name + ".npy";
    const std::vector<unsigned char> body = npy_bytes(arr);
    if (body.size() >= 0xFFFFFFFFull || zip.size() >= 0xFFFFFFFFull)
      throw std::runtime_error("npz: member larger than 4 GiB");
    const uint32_t crc = crc32_of(body.data(), body.size());
    const uint32_t offset = (uint32_t)zip.size();
    put32(zip, 0x04034b50u);  // local file header
    put16(zip, 20);           // version needed
    put16(zip, 0);            // flags
    put16(zip, 0);            // stored
    put16(zip, 0);            // time
    put16(zip, 0x21);         // date (1980-01-01)
    put32(zip, crc);
    put32(zip, (uint32_t)body.size());
    put32(zip, (uint32_t)body.size());
    put16(zip, (uint32_t)member.size());
    put16(zip, 0);
    zip.insert(zip.end(), member.begin(), member.end());
    zip.insert(zip.end(), body.begin(), body.end());
    put32(central, 0x02014b50u);  // central directory entry
    put16(central, 20);           // version made by
    put16(central, 20);
    put16(central, 0);
    put16(central, 0);
    put16(central, 0);
    put16(central, 0x21);
    put32(central, crc);
    put32(central, (uint32_t)body.size());
    put32(central, (uint32_t)body.size());
    put16(central, (uint32_t)member.size());
    put16(central, 0);  // extra
    put16(central, 0);  // comment
    put16(central, 0);  // disk
    put16(central, 0);  // internal attributes
    put32(central, 0);  // external attributes
    put32(central, offset);
    central.insert(central.end(), member.begin(), member.end());
    ++count;
  }
  const uint32_t cd_offset = (uint32_t)zip.size();
  zip.insert(zip.end(), central.begin(), central.end());
  put32(zip, 0x06054b50u);  // end of central directory
  put16(zip, 0);
  put16(zip, 0);
  put16(zip, count);
  put16(zip, count);
  put32(zip, (uint32_t)central.size());
  put32(zip, cd_offset);
  put16(zip, 0);
  FILE* f = std::fopen(file.c_str(), "wb");
  if (!f) throw std::runtime_error("Could not open '" + file + "' for writing");
  const size_t w = std::fwrite(zip.data(), 1, zip.size(), f);
  const int c = std::fclose(f);
  if (w != zip.size() || c != 0) throw std::runtime_error("Could not write '" + file + "'");
}

std::map<std::string, NpyArray> npz_read(const std::string& file) {
  FILE* f = std::fopen(file.c_str(), "rb");
  if (!f) throw std::runtime_error("Could not find '" + file + "'");
  std::vector<unsigned char> buf;
  unsigned char chunk[1 << 16];
  size_t r;
  while ((r = std::fread(chunk, 1, sizeof(chunk), f)) > 0) buf.insert(buf.end(), chunk, chunk + r);
  std::fclose(f);
  const size_t n = buf.size();
  // end of central directory: last occurrence of its signature (comment at most 64 KiB)
  size_t eocd = std::string::npos;
  for (long long i = (long long)n - 22; i >= 0 && (long long)n - i <= 22 + 65535; --i)
    if (get32(&buf[(size_t)i]) == 0x06054b50u) {
      eocd = (size_t)i;
      break;
    }
  if (eocd == std::string::npos || eocd + 22 > n)
    throw std::runtime_error("'" + file + "' is not a zip archive");
  const uint32_t entries = get16(&buf[eocd + 10]);
  size_t cd = get32(&buf[eocd + 16]);
  std::map<std::string, NpyArray> out;
  for (uint32_t e = 0; e < entries; ++e) {
    if (cd + 46 > n || get32(&buf[cd]) != 0x02014b50u)
      throw std::runtime_error("'" + file + "': damaged central directory");
    const uint32_t method = get16(&buf[cd + 10]);
    const uint32_t crc = get32(&buf[cd + 16]);
    const uint32_t csize = get32(&buf[cd + 20]);
    const uint32_t nlen = get16(&buf[cd + 28]), xlen = get16(&buf[cd + 30]),
                   clen = get16(&buf[cd + 32]);
    const size_t loc = get32(&buf[cd + 42]);  // offsets widened before any addition
    if (cd + 46 + (size_t)nlen > n)
      throw std::runtime_error("'" + file + "': damaged central directory");
    std::string name(reinterpret_cast<const char*>(&buf[cd + 46]), nlen);
    cd += 46 + (size_t)nlen + (size_t)xlen + (size_t)clen;
    if (loc + 30 > n || get32(&buf[loc]) != 0x04034b50u)
      throw std::runtime_error("'" + file + "': damaged member '" + name + "'");
    const size_t data = loc + 30 + (size_t)get16(&buf[loc + 26]) + (size_t)get16(&buf[loc + 28]);
    if (method != 0)
      throw std::runtime_error("'" + file + "': member '" + name + "' is compressed");
    if (data > n || (size_t)csize > n - data)
      throw std::runtime_error("'" + file + "': truncated member '" + name + "'");
    if (crc32_of(&buf[data], csize) != crc)
      throw std::runtime_error("'" + file + "': CRC mismatch in member '" + name + "'");
    if (name.size() > 4 && name.compare(name.size() - 4, 4, ".npy") == 0)
      name.resize(name.size() - 4);
    out[name] = npy_parse(&buf[data], csize, name);
  }
  return out;
}

}  // namespace tb
