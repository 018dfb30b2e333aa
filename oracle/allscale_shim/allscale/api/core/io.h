// Stand-in for allscale/api/core/io.h: FileIOManager backed by plain files in
// the working directory (cell.h:1367-1387, cell_test.cc:338-370).
// TEST INFRASTRUCTURE ONLY (oracle).
#pragma once

#include <fstream>
#include <memory>
#include <string>

namespace allscale {
namespace api {
namespace core {

struct Entry {
    std::string name;
};

class OutputStream {
    std::shared_ptr<std::ofstream> out_;

  public:
    explicit OutputStream(const std::string& name) : out_(std::make_shared<std::ofstream>(name)) {}
    template <typename T>
    OutputStream& operator<<(const T& v) {
        *out_ << v;
        return *this;
    }
    void close() { out_->close(); }
};

class InputStream {
    std::shared_ptr<std::ifstream> in_;

  public:
    explicit InputStream(const std::string& name) : in_(std::make_shared<std::ifstream>(name)) {}
    template <typename T>
    InputStream& operator>>(T& v) {
        *in_ >> v;
        return *this;
    }
    explicit operator bool() const { return static_cast<bool>(*in_); }
    void close() { in_->close(); }
};

class FileIOManager {
  public:
    static FileIOManager& getInstance() {
        static FileIOManager m;
        return m;
    }
    Entry createEntry(const std::string& name) { return {name}; }
    OutputStream openOutputStream(const Entry& e) { return OutputStream(e.name); }
    InputStream openInputStream(const Entry& e) { return InputStream(e.name); }
    void close(OutputStream& s) { s.close(); }
    void close(InputStream& s) { s.close(); }
};

}  // namespace core
}  // namespace api
}  // namespace allscale
