// A minimal writer of the HDF5 file format (no libhdf5 on the machines this library runs
// on): one root group holding attributes (32-bit integers, doubles, strings) and
// contiguous little-endian FP64 datasets, each with string attributes. The structures
// follow the published format specification: superblock version 0, version-1 object
// headers, a symbol-table group (version-1 B-tree, symbol-table node, local heap).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace tdg {

class H5Writer {
  public:
    void attr_int(const std::string &name, int32_t v);
    void attr_double(const std::string &name, double v);
    void attr_string(const std::string &name, const std::string &v);
    // dims in C order (slowest first); data holds prod(dims) values in that order.
    void dataset(const std::string &name, const std::vector<uint64_t> &dims, std::vector<double> data,
                 const std::string &unit, const std::string &dimensions);
    // Writes the file; returns 0 or TDG_ERR_IO / TDG_ERR_PARAM through set_error.
    int write(const std::string &path) const;

  private:
    struct Attr {
        std::string name;
        int kind;  // 0 int32, 1 double, 2 string
        int32_t i;
        double d;
        std::string s;
    };
    struct Dset {
        std::string name;
        std::vector<uint64_t> dims;
        std::vector<double> data;
        std::vector<Attr> attrs;
    };
    std::vector<Attr> root_attrs_;
    std::vector<Dset> dsets_;
};

}  // namespace tdg
