// Stand-in for <boost/filesystem.hpp>, backed by std::filesystem, used only to
// compile the reference's src/core/filesystem.cpp for the oracle build.
// Boost is not installed here; the reference uses only these calls
// (exists, path::{has_parent_path,parent_path,has_root_path,string},
// create_directory/ies, rename, remove, remove_all). No arithmetic involved.
#ifndef ORACLE_SHIM_BOOST_FILESYSTEM_HPP
#define ORACLE_SHIM_BOOST_FILESYSTEM_HPP
#include <filesystem>
#include <string>
namespace boost {
namespace filesystem {
using path = std::filesystem::path;
inline bool exists(const path &p) { std::error_code ec; return std::filesystem::exists(p, ec); }
inline bool create_directory(const path &p) { std::error_code ec; return std::filesystem::create_directory(p, ec); }
inline bool create_directories(const path &p) { std::error_code ec; return std::filesystem::create_directories(p, ec); }
inline void rename(const path &a, const path &b) { std::filesystem::rename(a, b); }
inline bool remove(const path &p) { std::error_code ec; return std::filesystem::remove(p, ec); }
inline unsigned long remove_all(const path &p) { std::error_code ec; return (unsigned long)std::filesystem::remove_all(p, ec); }
}  // namespace filesystem
}  // namespace boost
#endif
