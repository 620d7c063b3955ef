// Host execution shim of the Boost.Filesystem calls in the reference's
// Bubble constructor and utils.h (backup copies of its sources next to the
// output): every file operation is a no-op here.
#pragma once
#include <exception>
#include <string>
namespace boost {
namespace filesystem {
class path {
  public:
    path() {}
    path(const char* s) : s_(s) {}
    path(const std::string& s) : s_(s) {}
    std::string string() const { return s_; }
    path filename() const { return path(s_.substr(s_.find_last_of('/') + 1)); }
    path operator/(const path& o) const { return path(s_ + "/" + o.s_); }
  private:
    std::string s_;
};
enum class copy_option { none, fail_if_exists, overwrite_if_exists };
struct filesystem_error : std::exception {
    const char* what() const noexcept override { return "filesystem"; }
};
inline bool exists(const path&) { return false; }
inline bool is_directory(const path&) { return false; }
inline void remove_all(const path&) {}
inline bool create_directory(const path&) { return true; }
inline bool create_directories(const path&) { return true; }
inline void copy_file(const path&, const path&, copy_option = copy_option::none) {}
struct directory_entry {
    path p;
    const path& path_() const { return p; }
    filesystem::path path() const { return p; }
};
class directory_iterator {
  public:
    directory_iterator() {}
    explicit directory_iterator(const filesystem::path&) {}
    bool operator!=(const directory_iterator&) const { return false; }
    directory_iterator& operator++() { return *this; }
    const directory_entry* operator->() const { return &e_; }
  private:
    directory_entry e_;
};
}  // namespace filesystem
}  // namespace boost
