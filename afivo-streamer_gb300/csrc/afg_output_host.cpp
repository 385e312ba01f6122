// File formats of the output writers (see afg_output_host.h).
#include "afg_output_host.h"

#include <cmath>
#include <cstring>

namespace afg_out {

/* ---- VTK XML unstructured grid ----------------------------------------- */

VtuFile::~VtuFile() {
  if (f_) fclose(f_);
}

bool VtuFile::open(const std::string& path, double time, int cycle, long long n_points, long long n_cells,
                   const std::vector<VtuArray>& arrays) {
  f_ = fopen(path.c_str(), "wb");
  if (!f_) return false;
  // 4-byte size headers (the default of a version 0.1 file) unless an array
  // does not fit in them
  h64_ = false;
  for (const VtuArray& a : arrays)
    if (a.bytes > 0xffffffffull) h64_ = true;
  const uint64_t hb = h64_ ? 8 : 4;
  std::string x;
  char buf[512];
  x += "<?xml version=\"1.0\"?>\n";
  x += h64_ ? "<VTKFile type=\"UnstructuredGrid\" version=\"1.0\" byte_order=\"LittleEndian\" "
              "header_type=\"UInt64\">\n"
            : "<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n";
  x += "  <UnstructuredGrid>\n";
  x += "    <FieldData>\n";
  snprintf(buf, sizeof(buf),
           "      <DataArray type=\"Float64\" Name=\"TIME\" NumberOfTuples=\"1\" format=\"ascii\">\n"
           "        %.17g\n      </DataArray>\n",
           time);
  x += buf;
  snprintf(buf, sizeof(buf),
           "      <DataArray type=\"Int32\" Name=\"CYCLE\" NumberOfTuples=\"1\" format=\"ascii\">\n"
           "        %d\n      </DataArray>\n",
           cycle);
  x += buf;
  x += "    </FieldData>\n";
  snprintf(buf, sizeof(buf), "    <Piece NumberOfPoints=\"%lld\" NumberOfCells=\"%lld\">\n", n_points, n_cells);
  x += buf;
  uint64_t off = 0;
  std::string open_sec;
  for (const VtuArray& a : arrays) {
    if (a.section != open_sec) {
      if (!open_sec.empty()) x += "      </" + open_sec + ">\n";
      x += "      <" + a.section + ">\n";
      open_sec = a.section;
    }
    snprintf(buf, sizeof(buf),
             "        <DataArray type=\"%s\" Name=\"%s\" NumberOfComponents=\"%d\" format=\"appended\" "
             "offset=\"%llu\"/>\n",
             a.xml_type.c_str(), a.name.c_str(), a.ncomp, (unsigned long long)off);
    x += buf;
    off += hb + a.bytes;
  }
  if (!open_sec.empty()) x += "      </" + open_sec + ">\n";
  x += "    </Piece>\n";
  x += "  </UnstructuredGrid>\n";
  x += "  <AppendedData encoding=\"raw\">\n_";
  return fwrite(x.data(), 1, x.size(), f_) == x.size();
}

bool VtuFile::begin(uint64_t bytes) {
  if (h64_) return fwrite(&bytes, 8, 1, f_) == 1;
  const uint32_t b = (uint32_t)bytes;
  return fwrite(&b, 4, 1, f_) == 1;
}

bool VtuFile::write(const void* data, size_t bytes) {
  return bytes == 0 || fwrite(data, 1, bytes, f_) == bytes;
}

bool VtuFile::close() {
  if (!f_) return false;
  const char* tail = "\n  </AppendedData>\n</VTKFile>\n";
  bool ok = fwrite(tail, 1, strlen(tail), f_) == strlen(tail);
  ok = (fclose(f_) == 0) && ok;
  f_ = nullptr;
  return ok;
}

/* ---- Fortran Ew.d ------------------------------------------------------- */

std::string fortran_e(double v, int w, int d) {
  std::string s;
  if (std::isnan(v)) {
    s = "NaN";
  } else if (std::isinf(v)) {
    s = v < 0 ? "-Infinity" : "Infinity";
  } else {
    // d significant digits, correctly rounded: d1.d2...dd E x; the Fortran
    // form is 0.d1d2...dd with exponent x + 1 (zero has exponent 0)
    char buf[64];
    snprintf(buf, sizeof(buf), "%.*E", d - 1, std::fabs(v));
    std::string digits;
    const char* p = buf;
    for (; *p && *p != 'E'; p++)
      if (*p >= '0' && *p <= '9') digits += *p;
    int e = (*p == 'E') ? atoi(p + 1) : 0;
    if (v != 0.0) e += 1;
    s = std::signbit(v) ? "-0." : "0.";
    s += digits;
    char eb[16];
    const int ae = e < 0 ? -e : e;
    if (ae <= 99)
      snprintf(eb, sizeof(eb), "E%c%02d", e < 0 ? '-' : '+', ae);
    else
      snprintf(eb, sizeof(eb), "%c%03d", e < 0 ? '-' : '+', ae);
    s += eb;
  }
  if ((int)s.size() > w) return std::string(w, '*');
  return std::string(w - s.size(), ' ') + s;
}

/* ---- .npy --------------------------------------------------------------- */

std::string npy_header(const char* descr, const std::vector<long long>& shape) {
  std::string dict = std::string("{'descr': '") + descr + "', 'fortran_order': True, 'shape': (";
  for (size_t i = 0; i < shape.size(); i++) {
    dict += std::to_string(shape[i]);
    if (i + 1 < shape.size() || shape.size() == 1) dict += ",";
    if (i + 1 < shape.size()) dict += " ";
  }
  dict += "), }";
  // magic (6) + version (2) + length (2) + dict + padding + '\n', a multiple of 64
  size_t total = 10 + dict.size() + 1;
  total = (total + 63) / 64 * 64;
  dict += std::string(total - 10 - dict.size() - 1, ' ');
  dict += '\n';
  const uint16_t len = (uint16_t)dict.size();
  std::string h("\x93NUMPY\x01\x00", 8);
  h += (char)(len & 0xff);
  h += (char)(len >> 8);
  return h + dict;
}

/* ---- zip (stored) ------------------------------------------------------- */

uint32_t crc32_update(uint32_t crc, const void* data, size_t n) {
  static uint32_t table[256];
  static bool init = false;
  if (!init) {
    for (uint32_t i = 0; i < 256; i++) {
      uint32_t c = i;
      for (int k = 0; k < 8; k++) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
      table[i] = c;
    }
    init = true;
  }
  const unsigned char* p = static_cast<const unsigned char*>(data);
  crc = ~crc;
  for (size_t i = 0; i < n; i++) crc = table[(crc ^ p[i]) & 0xff] ^ (crc >> 8);
  return ~crc;
}

static void put16(std::string& s, uint32_t v) {
  s += (char)(v & 0xff);
  s += (char)((v >> 8) & 0xff);
}
static void put32(std::string& s, uint32_t v) {
  put16(s, v & 0xffff);
  put16(s, v >> 16);
}

ZipStore::~ZipStore() {
  if (f_) fclose(f_);
}

bool ZipStore::open(const std::string& path) {
  f_ = fopen(path.c_str(), "wb");
  pos_ = 0;
  entries_.clear();
  return f_ != nullptr;
}

bool ZipStore::add(const std::string& name, const std::string& data) {
  if (!f_ || data.size() > 0xfffffffeull || pos_ > 0xfffffffeull) return false;
  Entry e{name, crc32_update(0, data.data(), data.size()), (uint32_t)data.size(), (uint32_t)pos_};
  std::string h;
  put32(h, 0x04034b50u);
  put16(h, 10);  // version needed: 1.0 (stored)
  put16(h, 0);   // flags
  put16(h, 0);   // method: stored
  put16(h, 0);   // time
  put16(h, 0x21);  // date: 1980-01-01
  put32(h, e.crc);
  put32(h, e.size);
  put32(h, e.size);
  put16(h, (uint32_t)name.size());
  put16(h, 0);
  h += name;
  if (fwrite(h.data(), 1, h.size(), f_) != h.size()) return false;
  if (!data.empty() && fwrite(data.data(), 1, data.size(), f_) != data.size()) return false;
  pos_ += h.size() + data.size();
  entries_.push_back(e);
  return true;
}

bool ZipStore::close() {
  if (!f_) return false;
  std::string c;
  for (const Entry& e : entries_) {
    put32(c, 0x02014b50u);
    put16(c, 20);  // made by
    put16(c, 10);  // needed
    put16(c, 0);
    put16(c, 0);
    put16(c, 0);
    put16(c, 0x21);
    put32(c, e.crc);
    put32(c, e.size);
    put32(c, e.size);
    put16(c, (uint32_t)e.name.size());
    put16(c, 0);  // extra
    put16(c, 0);  // comment
    put16(c, 0);  // disk
    put16(c, 0);  // internal attributes
    put32(c, 0);  // external attributes
    put32(c, e.offset);
    c += e.name;
  }
  std::string end;
  put32(end, 0x06054b50u);
  put16(end, 0);
  put16(end, 0);
  put16(end, (uint32_t)entries_.size());
  put16(end, (uint32_t)entries_.size());
  put32(end, (uint32_t)c.size());
  put32(end, (uint32_t)pos_);
  put16(end, 0);
  bool ok = fwrite(c.data(), 1, c.size(), f_) == c.size() && fwrite(end.data(), 1, end.size(), f_) == end.size();
  ok = (fclose(f_) == 0) && ok;
  f_ = nullptr;
  return ok;
}

}  // namespace afg_out
