/*
 * H5File.h -- the output side of the reference's main.cc (source/main.cc:56-89) without
 * HighFive, xtensor-io or libhdf5: an RAII handle over sayram_h5.h.
 *
 *   HighFive::File file(filename, HighFive::File::Overwrite);  ->  sayram::H5File file(filename);
 *   xt::dump(file, "/f/0", solver.f(), xt::dump_mode::overwrite) ->  file.dump("/f/0", solver.f());
 *   xt::dump(file, "/alpha0", alpha0, ...)  (an Eigen vector)     ->  file.dump("/alpha0", alpha0.data(), {n});
 *
 * dump() of an array type takes anything with data() and shape() in C order (xtensor); the
 * pointer form takes the dimensions explicitly. Errors throw std::runtime_error with the
 * library's message. The file is complete when the object is destroyed or close() returns.
 */
#ifndef SAYRAM_H5FILE_H
#define SAYRAM_H5FILE_H

#include <stdexcept>
#include <string>
#include <vector>

#include "sayram_h5.h"

namespace sayram {

class H5File {
 public:
  explicit H5File(const std::string& path) { check(sayram_h5_create(path.c_str(), &h_), "sayram_h5_create"); }
  ~H5File() {
    if (h_) sayram_h5_close(h_);
  }
  H5File(const H5File&) = delete;
  H5File& operator=(const H5File&) = delete;

  void dump(const std::string& path, const double* data, const std::vector<long long>& dims) {
    check(sayram_h5_write(h_, path.c_str(), data, (int)dims.size(), dims.data()), "sayram_h5_write");
  }
  template <class Array>
  void dump(const std::string& path, const Array& a) {
    std::vector<long long> dims;
    for (auto d : a.shape()) dims.push_back((long long)d);
    dump(path, a.data(), dims);
  }
  void close() {
    sayram_h5 h = h_;
    h_ = nullptr;
    if (h) check(sayram_h5_close(h), "sayram_h5_close");
  }

 private:
  sayram_h5 h_ = nullptr;
  static void check(int rc, const char* what) {
    if (rc != SAYRAM_OK) throw std::runtime_error(std::string(what) + ": " + sayram_last_error());
  }
};

}  // namespace sayram

#endif /* SAYRAM_H5FILE_H */
