// Stand-in for boost/property_tree/json_parser.hpp.  The oracle harness never
// parses parameter files, so reading raises ptree_error; writing emits a flat,
// human-readable dump that is only used for diagnostics.
#pragma once
#include <fstream>
#include <istream>
#include <ostream>
#include "ptree.hpp"

namespace boost {
namespace property_tree {

inline void read_json(std::istream&, ptree&) { throw ptree_error("JSON input is not supported by the oracle shim"); }
inline void read_json(const std::string& file, ptree&) {
    throw ptree_error("JSON input is not supported by the oracle shim: " + file);
}
inline void write_json_rec(std::ostream& os, const ptree& pt, int depth) {
    for (ptree::const_iterator it = pt.begin(); it != pt.end(); ++it) {
        os << std::string(2 * depth, ' ') << '"' << it->first << "\": \"" << it->second.data() << "\"\n";
        write_json_rec(os, it->second, depth + 1);
    }
}
inline void write_json(std::ostream& os, const ptree& pt, bool = true) { write_json_rec(os, pt, 0); }
inline void write_json(const std::string& file, const ptree& pt, const std::locale& = std::locale(), bool = true) {
    std::ofstream os(file.c_str());
    write_json_rec(os, pt, 0);
}

}  // namespace property_tree
}  // namespace boost
