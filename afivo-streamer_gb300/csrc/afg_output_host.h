// File formats of the output writers (host side).  The device gathers and
// interpolates (afg_output.cuh); these routines only put bytes into files.
//
//   VtuFile     VTK XML unstructured grid with appended raw data, the layout
//               af_write_vtk writes (afivo/src/m_af_output.f90:556-752,
//               afivo/src/m_vtk.f90): FieldData TIME/CYCLE, Float32 points,
//               Int32 connectivity/offsets/types, Float64 cell data
//   fortran_e   Fortran Ew.d edit descriptor (af_write_plane's E20.8)
//   npy_header  .npy version 1.0 header of a Fortran-ordered array (m_npy.f90)
//   ZipStore    uncompressed .zip archive (what `zip -q0` makes; .npz files)
#pragma once

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

namespace afg_out {

// One appended array of a .vtu file: its XML element and its size in bytes.
struct VtuArray {
  std::string section;  // "Points", "Cells" or "CellData"
  std::string xml_type; // "Float32", "Int32", "Float64"
  std::string name;
  int ncomp;
  uint64_t bytes;
};

class VtuFile {
 public:
  ~VtuFile();
  // Writes the XML part (offsets of every appended array follow from the
  // sizes) and opens the appended section.  Returns false on an I/O error.
  bool open(const std::string& path, double time, int cycle, long long n_points, long long n_cells,
            const std::vector<VtuArray>& arrays);
  // the arrays in the order given to open(): begin() writes the size
  // header, write() appends raw bytes (any number of calls per array)
  bool begin(uint64_t bytes);
  bool write(const void* data, size_t bytes);
  bool close();
  bool header64() const { return h64_; }

 private:
  FILE* f_ = nullptr;
  bool h64_ = false;
};

// Fortran Ew.d output of one value (width w, d digits after the point,
// mantissa in [0.1, 1), two-digit exponent with E, three digits without it)
std::string fortran_e(double v, int w, int d);

// .npy (version 1.0) header for a little-endian array in Fortran order
std::string npy_header(const char* descr, const std::vector<long long>& shape);

// CRC-32 (IEEE 802.3 polynomial, reflected, table driven) as used by zip
uint32_t crc32_update(uint32_t crc, const void* data, size_t n);

// Stored (method 0) zip archive written entry by entry
class ZipStore {
 public:
  ~ZipStore();
  bool open(const std::string& path);
  bool add(const std::string& name, const std::string& data);
  bool close();

 private:
  struct Entry {
    std::string name;
    uint32_t crc, size, offset;
  };
  FILE* f_ = nullptr;
  uint64_t pos_ = 0;
  std::vector<Entry> entries_;
};

}  // namespace afg_out
