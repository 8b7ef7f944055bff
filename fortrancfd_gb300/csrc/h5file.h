// HDF5 files of the reference's output and restart (SRC/write_hdf5.f90,
// SRC/read_hdf5.f90), written and read here from the published HDF5 file
// format (superblock version 0, version-1 object headers, symbol-table
// groups with a version-1 B-tree, a local heap and symbol-table nodes,
// contiguous datasets, version-1 attribute messages): the layout libhdf5
// writes with its default ("earliest") format settings, which the
// reference's Fortran calls use. No HDF5 library is involved.
#pragma once

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

namespace edyn {

// The step group name of write_hdf5_b: Fortran's ("nout",i6.6,"_time",e11.5)
// (SRC/write_hdf5.f90:168), e.g. nout000012_time0.12000E-03.
std::string step_group_name(int nout, double time);

// One attribute of a step group: a rank-1, one-element array of float64
// (H5T_NATIVE_DOUBLE) or int32 (H5T_NATIVE_INTEGER), as write_hdf5_b
// creates them.
struct H5Attr {
  std::string name;
  bool is_int = false;
  double value = 0.0;
};

// A file being written: groups are appended below the root group, each
// with its rank-1 float64 datasets and its attributes. Every append writes
// the new raw data and metadata at the end of the file, then rewrites the
// root group's index and the superblock, so the file is readable after
// each append.
class H5Writer {
 public:
  H5Writer() = default;
  ~H5Writer();
  H5Writer(const H5Writer&) = delete;
  H5Writer& operator=(const H5Writer&) = delete;
  // truncates or creates the file; false (and err) on failure
  bool create(const std::string& path, std::string& err);
  // appends the group `name` with datasets rows[r * n .. r * n + n) named
  // row_names[r] and the attributes; names must be unique within the group
  bool add_group(const std::string& name, const std::vector<H5Attr>& attrs, const std::vector<std::string>& row_names,
                 const double* rows, int64_t n, std::string& err);
  bool close(std::string& err);
  bool is_open() const { return f_ != nullptr; }
  const std::string& path() const { return path_; }

 private:
  struct Entry {
    std::string name;
    uint64_t ohdr = 0;
    bool group = false;
    uint64_t btree = 0, heap = 0;  // group entries: their symbol table
  };
  uint64_t append(const std::vector<uint8_t>& bytes);
  bool write_symbol_table(std::vector<Entry> entries, uint64_t& btree, uint64_t& heap, std::string& err);
  bool rewrite_superblock(std::string& err);
  std::FILE* f_ = nullptr;
  std::string path_;
  uint64_t eof_ = 0;
  std::vector<Entry> root_;  // the step groups written so far
  uint64_t root_ohdr_ = 0, root_btree_ = 0, root_heap_ = 0;
  bool ok_ = true;
};

// A dataset or attribute value read back: float64 / integer data as doubles.
struct H5Value {
  std::vector<uint64_t> dims;
  std::vector<double> data;
  bool is_string = false;
  std::string text;
};

struct H5Object {
  std::string name;
  bool group = false;
  uint64_t ohdr = 0;
};

// Reads files in the layout above (superblock versions 0 and 1, version-1
// object headers with continuation blocks, symbol-table groups at any
// B-tree depth; dataspace versions 1 and 2; float32/64, signed and
// unsigned 8-64 bit integers and fixed-length strings in either byte order;
// contiguous and compact layouts, versions 1-3; attribute messages,
// versions 1-3). Paths are '/'-separated, relative to the root group.
class H5Reader {
 public:
  H5Reader() = default;
  ~H5Reader();
  H5Reader(const H5Reader&) = delete;
  H5Reader& operator=(const H5Reader&) = delete;
  bool open(const std::string& path, std::string& err);
  // members of a group in the group's name order (libhdf5's index order)
  bool list(const std::string& group, std::vector<H5Object>& out, std::string& err);
  bool read_dataset(const std::string& path, H5Value& v, std::string& err);
  bool read_attr(const std::string& object, const std::string& name, H5Value& v, std::string& err);
  bool attr_names(const std::string& object, std::vector<std::string>& out, std::string& err);

 private:
  struct Msg {
    uint16_t type;
    uint8_t flags;
    std::vector<uint8_t> data;
  };
  bool read_at(uint64_t addr, size_t len, std::vector<uint8_t>& out, std::string& err);
  bool header(uint64_t addr, std::vector<Msg>& msgs, std::string& err);
  bool group_members(uint64_t ohdr, std::vector<H5Object>& out, std::string& err);
  bool btree_walk(uint64_t addr, const std::vector<uint8_t>& heap, std::vector<H5Object>& out, int depth,
                  std::string& err);
  bool resolve(const std::string& path, uint64_t& ohdr, std::string& err);
  std::FILE* fp_ = nullptr;
  uint64_t size_ = 0;
  uint64_t base_ = 0;
  uint64_t root_ohdr_ = 0;
  int leaf_k_ = 4, internal_k_ = 16;
};

}  // namespace edyn
