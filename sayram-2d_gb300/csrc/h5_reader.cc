// h5_reader.cc -- the input side of the reference's HDF5 use: xt::load_hdf5 of one dataset, and
// the Albert_Young D table (Albert_Young_IO::read_D, source/Cases/Albert_Young_IO.cc:17-36).
//
// libhdf5 is not a dependency: this reads the classic subset of the HDF5 file format that
// libhdf5 writes by default (and h5py with its default library-version bounds):
//   * superblock version 0 or 1 (any user block of 512 * 2^k bytes), 8-byte addresses/lengths;
//   * groups as symbol tables: version-1 B-trees (any depth) of symbol-table nodes, names in a
//     local heap;
//   * version-1 object headers with continuation blocks;
//   * datasets of IEEE binary32/binary64 in either byte order, dataspace version 1 or 2, data
//     layout versions 1-3 with contiguous or compact storage (unallocated storage reads as 0).
// Anything else -- superblock 2/3, version-2 object headers, link-message groups, chunked or
// filtered storage, other datatypes -- is refused with a message saying what was found.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "host_errors.h"
#include "sayram_gpu.h"
#include "sayram_h5.h"

namespace {

constexpr uint64_t kUndef = ~0ull;

struct Bad {  // a format error, with its message
  std::string msg;
};

class File {
 public:
  explicit File(const char* path) : fp_(std::fopen(path, "rb")) {
    if (!fp_) throw Bad{std::string("cannot open ") + path};
    std::fseek(fp_, 0, SEEK_END);
    size_ = (uint64_t)std::ftell(fp_);
    find_superblock();
  }
  ~File() {
    if (fp_) std::fclose(fp_);
  }
  File(const File&) = delete;
  File& operator=(const File&) = delete;

  // object header address of the object at an absolute path ("/a/b")
  uint64_t locate(const std::string& path) {
    uint64_t obj = root_;
    size_t p = 0;
    while (p < path.size()) {
      while (p < path.size() && path[p] == '/') ++p;
      size_t e = path.find('/', p);
      if (e == std::string::npos) e = path.size();
      if (e > p) obj = lookup(obj, path.substr(p, e - p));
      p = e;
    }
    return obj;
  }

  struct Data {
    std::vector<long long> dims;
    std::vector<double> v;
  };

  Data read_dataset(uint64_t ohdr, const std::string& name) {
    std::vector<Msg> msgs = messages(ohdr);
    const Msg *space = nullptr, *type = nullptr, *layout = nullptr;
    for (const Msg& m : msgs) {
      if (m.type == 0x1) space = &m;
      if (m.type == 0x3) type = &m;
      if (m.type == 0x8) layout = &m;
      if (m.type == 0xB) throw Bad{name + ": filtered (compressed) storage is not supported"};
      if (m.type == 0x11) throw Bad{name + " is a group, not a dataset"};
    }
    if (!space || !type || !layout) throw Bad{name + ": not a dataset (dataspace/datatype/layout missing)"};
    Data d;
    // dataspace
    const std::vector<uint8_t>& sb = space->body;
    need(sb.size() >= 4, name + ": dataspace message");
    const int sver = sb[0], rank = sb[1];
    need(sver == 1 || sver == 2, name + ": dataspace version " + std::to_string(sver));
    if (sver == 2 && sb[3] == 2) rank_null(name);  // null dataspace
    const size_t doff = sver == 1 ? 8 : 4;
    need(sb.size() >= doff + 8 * (size_t)rank, name + ": dataspace message");
    uint64_t n = 1;
    for (int k = 0; k < rank; ++k) {
      const uint64_t v = le64(&sb[doff + 8 * k]);
      need(v < (1ull << 48) && (v == 0 || n <= (1ull << 60) / v), name + ": dataspace dimensions out of range");
      d.dims.push_back((long long)v);
      n *= v;
    }
    // datatype
    const std::vector<uint8_t>& tb = type->body;
    need(tb.size() >= 8, name + ": datatype message");
    const int cls = tb[0] & 0x0f;
    const bool big = tb[1] & 1;
    const uint32_t esz = le32(&tb[4]);
    if (cls != 1 || (esz != 4 && esz != 8))
      throw Bad{name + ": datatype class " + std::to_string(cls) + " size " + std::to_string(esz) +
                " (only IEEE binary32/binary64 is read)"};
    // layout
    const std::vector<uint8_t>& lb = layout->body;
    need(lb.size() >= 2, name + ": layout message");
    const int lver = lb[0];
    std::vector<uint8_t> raw;
    const uint64_t bytes = n * esz;
    // storage that was never written reads as zeros, but only up to the size of the file itself
    need(bytes <= std::max<uint64_t>(size_, 1ull << 20) * 8, name + ": dataset larger than its file allows");
    if (lver == 3) {
      const int lcls = lb[1];
      if (lcls == 1) {
        need(lb.size() >= 18, name + ": layout message");
        const uint64_t addr = le64(&lb[2]), sz = le64(&lb[10]);
        need(addr == kUndef || sz == bytes, name + ": contiguous size differs from the dataspace");
        raw = addr == kUndef ? std::vector<uint8_t>(bytes, 0) : read(base_ + addr, bytes);
      } else if (lcls == 0) {
        need(lb.size() >= 4, name + ": layout message");
        const uint32_t sz = (uint32_t)lb[2] | ((uint32_t)lb[3] << 8);
        need(sz == bytes && lb.size() >= 4 + (size_t)sz, name + ": compact size differs from the dataspace");
        raw.assign(lb.begin() + 4, lb.begin() + 4 + sz);
      } else {
        throw Bad{name + ": chunked storage is not supported (write it contiguous)"};
      }
    } else if (lver == 1 || lver == 2) {
      need(lb.size() >= 16, name + ": layout message");
      const int lcls = lb[2];
      if (lcls != 1) throw Bad{name + ": layout class " + std::to_string(lcls) + " is not supported"};
      const uint64_t addr = le64(&lb[8]);
      raw = addr == kUndef ? std::vector<uint8_t>(bytes, 0) : read(base_ + addr, bytes);
    } else {
      throw Bad{name + ": layout version " + std::to_string(lver)};
    }
    d.v.resize(n);
    for (uint64_t k = 0; k < n; ++k) {
      uint8_t b[8];
      for (uint32_t q = 0; q < esz; ++q) b[q] = raw[k * esz + (big ? esz - 1 - q : q)];
      if (esz == 8) {
        uint64_t u = le64(b);
        std::memcpy(&d.v[k], &u, 8);
      } else {
        uint32_t u = le32(b);
        float f;
        std::memcpy(&f, &u, 4);
        d.v[k] = f;
      }
    }
    return d;
  }

 private:
  struct Msg {
    unsigned type;
    std::vector<uint8_t> body;
  };
  FILE* fp_;
  uint64_t size_ = 0, base_ = 0, root_ = kUndef;
  long visits_ = 0;  // B-tree nodes read by this file's lookups

  static uint64_t le64(const uint8_t* p) {
    uint64_t v = 0;
    for (int k = 7; k >= 0; --k) v = (v << 8) | p[k];
    return v;
  }
  static uint32_t le32(const uint8_t* p) { return (uint32_t)p[0] | (uint32_t)p[1] << 8 | (uint32_t)p[2] << 16 | (uint32_t)p[3] << 24; }
  static uint16_t le16(const uint8_t* p) { return (uint16_t)(p[0] | p[1] << 8); }
  static void need(bool ok, const std::string& what) {
    if (!ok) throw Bad{"malformed HDF5 file: " + what};
  }
  [[noreturn]] static void rank_null(const std::string& name) { throw Bad{name + ": null dataspace"}; }

  std::vector<uint8_t> read(uint64_t off, uint64_t n) {
    need(off <= size_ && n <= size_ - off, "a structure runs past the end of the file");
    std::vector<uint8_t> out(n);
    if (n && (std::fseek(fp_, (long)off, SEEK_SET) != 0 || std::fread(out.data(), 1, n, fp_) != n))
      throw Bad{"read error"};
    return out;
  }

  void find_superblock() {
    static const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    for (uint64_t off = 0; off + 8 <= size_; off = off ? off * 2 : 512) {
      std::vector<uint8_t> s = read(off, 8);
      if (std::memcmp(s.data(), sig, 8)) continue;
      std::vector<uint8_t> h = read(off, std::min<uint64_t>(size_ - off, 128));
      need(h.size() >= 24, "superblock");
      const int ver = h[8];
      if (ver > 1)
        throw Bad{"HDF5 superblock version " + std::to_string(ver) +
                  " (only the classic versions 0 and 1 are read; write the file with h5py's default or "
                  "libver='earliest')"};
      need(h[13] == 8 && h[14] == 8, "only 8-byte offsets and lengths are read");
      size_t p = 24 + (ver == 1 ? 4 : 0);
      need(h.size() >= p + 32 + 40, "superblock");
      base_ = le64(&h[p]);
      need(base_ == off, "base address differs from the superblock's position");
      root_ = le64(&h[p + 32 + 8]);  // root group symbol table entry: object header address
      return;
    }
    throw Bad{"not an HDF5 file (no signature at 0, 512, 1024, ...)"};
  }

  std::vector<Msg> messages(uint64_t addr) {
    std::vector<uint8_t> h = read(base_ + addr, 16);
    if (h[0] != 1) {
      if (!std::memcmp(h.data(), "OHDR", 4))
        throw Bad{"version-2 object headers are not read (write the file with libver='earliest')"};
      need(false, "object header version " + std::to_string(h[0]));
    }
    const unsigned nmsg = le16(&h[2]);
    std::vector<std::pair<uint64_t, uint64_t>> blocks{{base_ + addr + 16, le32(&h[8])}};
    std::vector<Msg> out;
    for (size_t bi = 0; bi < blocks.size(); ++bi) {
      need(bi < 1024, "too many object header continuation blocks");
      std::vector<uint8_t> blk = read(blocks[bi].first, blocks[bi].second);
      size_t p = 0;
      while (p + 8 <= blk.size()) {
        const unsigned type = le16(&blk[p]), sz = le16(&blk[p + 2]);
        need(p + 8 + sz <= blk.size(), "message runs past its object header block");
        Msg m{type, std::vector<uint8_t>(blk.begin() + p + 8, blk.begin() + p + 8 + sz)};
        if (type == 0x10) {
          need(sz >= 16, "continuation message");
          blocks.push_back({base_ + le64(&m.body[0]), le64(&m.body[8])});
        }
        out.push_back(std::move(m));
        p += 8 + sz;
      }
    }
    need(out.size() == nmsg, "object header message count");
    return out;
  }

  // the child `name` of the group whose object header is at `grp`
  uint64_t lookup(uint64_t grp, const std::string& name) {
    uint64_t bt = kUndef, hp = kUndef;
    bool links = false;
    for (const Msg& m : messages(grp)) {
      if (m.type == 0x11 && m.body.size() >= 16) {
        bt = le64(&m.body[0]);
        hp = le64(&m.body[8]);
      }
      if (m.type == 0x6 || m.type == 0x2) links = true;
    }
    if (bt == kUndef) {
      if (links) throw Bad{"link-message groups are not read (write the file with libver='earliest')"};
      throw Bad{"'" + name + "': its parent is not a group"};
    }
    std::vector<uint8_t> hh = read(base_ + hp, 32);
    need(!std::memcmp(hh.data(), "HEAP", 4) && hh[4] == 0, "local heap");
    const std::vector<uint8_t> heap = read(base_ + le64(&hh[24]), le64(&hh[8]));
    uint64_t found = kUndef;
    search(bt, heap, name, &found, 0);
    if (found == kUndef) throw Bad{"no object named '" + name + "'"};
    return found;
  }

  std::string heap_str(const std::vector<uint8_t>& heap, uint64_t off) {
    need(off < heap.size(), "name offset outside the local heap");
    const uint8_t* s = &heap[off];
    const void* z = std::memchr(s, 0, heap.size() - off);
    need(z != nullptr, "unterminated name in the local heap");
    return std::string((const char*)s, (const char*)z);
  }

  void search(uint64_t node, const std::vector<uint8_t>& heap, const std::string& name, uint64_t* found, int depth) {
    need(depth < 64, "B-tree too deep");
    need(++visits_ < (1 << 20), "B-tree has too many nodes (a cycle?)");
    std::vector<uint8_t> h = read(base_ + node, 24);
    need(!std::memcmp(h.data(), "TREE", 4) && h[4] == 0, "group B-tree node");
    const int level = h[5];
    const unsigned used = le16(&h[6]);
    std::vector<uint8_t> kc = read(base_ + node + 24, (uint64_t)used * 16 + 8);
    for (unsigned c = 0; c < used && *found == kUndef; ++c) {
      const uint64_t child = le64(&kc[16 * c + 8]);
      if (level > 0) {
        search(child, heap, name, found, depth + 1);
        continue;
      }
      std::vector<uint8_t> sh = read(base_ + child, 8);
      need(!std::memcmp(sh.data(), "SNOD", 4) && sh[4] == 1, "symbol-table node");
      const unsigned nsym = le16(&sh[6]);
      std::vector<uint8_t> ents = read(base_ + child + 8, (uint64_t)nsym * 40);
      for (unsigned e = 0; e < nsym; ++e)
        if (heap_str(heap, le64(&ents[40 * e])) == name) {
          *found = le64(&ents[40 * e + 8]);
          break;
        }
    }
  }
};

int read_into(const char* file, const char* path, File::Data* out) {
  try {
    File f(file);
    *out = f.read_dataset(f.locate(path), path);
    return SAYRAM_OK;
  } catch (const Bad& b) {
    return sg::host_fail(SAYRAM_ERR_IO, std::string(file) + ": " + b.msg);
  } catch (const std::bad_alloc&) {
    return sg::host_fail(SAYRAM_ERR_OOM, "HDF5 input: out of host memory");
  }
}

double* copy_out(const std::vector<double>& v) {
  double* p = (double*)std::malloc(sizeof(double) * (v.empty() ? 1 : v.size()));
  if (p && !v.empty()) std::memcpy(p, v.data(), sizeof(double) * v.size());
  return p;
}

}  // namespace

extern "C" {

int sayram_h5_read(const char* file, const char* path, int max_rank, int* rank, long long* dims, double** data) {
  if (!file || !path || !rank || !data || (max_rank > 0 && !dims) || max_rank < 0)
    return sg::host_fail(SAYRAM_ERR_ARG, "sayram_h5_read: null argument");
  *data = nullptr;
  File::Data d;
  int rc = read_into(file, path, &d);
  if (rc) return rc;
  if ((int)d.dims.size() > max_rank)
    return sg::host_fail(SAYRAM_ERR_ARG, std::string("sayram_h5_read: ") + path + " has rank " +
                                             std::to_string(d.dims.size()) + " > max_rank");
  *rank = (int)d.dims.size();
  for (size_t k = 0; k < d.dims.size(); ++k) dims[k] = d.dims[k];
  *data = copy_out(d.v);
  if (!*data) return sg::host_fail(SAYRAM_ERR_OOM, "sayram_h5_read: out of host memory");
  return SAYRAM_OK;
}

void sayram_h5_free(void* p) { std::free(p); }

int sayram_dtable_load_h5(const char* file, sayram_dtable* out) {
  if (!file || !out) return sg::host_fail(SAYRAM_ERR_ARG, "sayram_dtable_load_h5: null argument");
  std::memset(out, 0, sizeof(*out));
  File::Data a, e, daa, dap, dpp;
  int rc;
  if ((rc = read_into(file, "/alpha0", &a)) || (rc = read_into(file, "/E", &e)) ||
      (rc = read_into(file, "/Daa", &daa)) || (rc = read_into(file, "/Dap", &dap)) ||
      (rc = read_into(file, "/Dpp", &dpp)))
    return rc;
  const long long na = (long long)a.v.size(), ne = (long long)e.v.size();
  if (a.dims.size() > 2 || e.dims.size() > 2 || na < 2 || ne < 2)
    return sg::host_fail(SAYRAM_ERR_ARG, std::string(file) + ": /alpha0 and /E must be vectors of >= 2 nodes");
  for (const File::Data* t : {&daa, &dap, &dpp})
    if (t->dims.size() != 2 || t->dims[0] != na || t->dims[1] != ne)
      return sg::host_fail(SAYRAM_ERR_ARG, std::string(file) + ": /Daa, /Dap, /Dpp must be (n_alpha0, n_E) = (" +
                                               std::to_string(na) + ", " + std::to_string(ne) + ")");
  out->n_alpha = (int)na;
  out->n_energy = (int)ne;
  out->alpha0_deg = copy_out(a.v);
  out->energy = copy_out(e.v);
  out->Daa = copy_out(daa.v);
  out->Dap = copy_out(dap.v);
  out->Dpp = copy_out(dpp.v);
  if (!out->alpha0_deg || !out->energy || !out->Daa || !out->Dap || !out->Dpp) {
    sayram_dtable_free(out);
    return sg::host_fail(SAYRAM_ERR_OOM, "sayram_dtable_load_h5: out of host memory");
  }
  return SAYRAM_OK;
}

void sayram_dtable_free(sayram_dtable* t) {
  if (!t) return;
  std::free((void*)t->alpha0_deg);
  std::free((void*)t->energy);
  std::free((void*)t->Daa);
  std::free((void*)t->Dap);
  std::free((void*)t->Dpp);
  std::memset(t, 0, sizeof(*t));
}

}  // extern "C"
