// h5_writer.cc -- the run's output file in HDF5, the format the reference writes through
// HighFive + xtensor-io (main.cc:57-89): /alpha0, /logEN, /f/<k> and /t, little-endian FP64.
//
// libhdf5 is not a dependency: this writer emits the classic subset of the HDF5 file format
// (format specification, superblock version 0) that libhdf5 itself writes by default and reads
// in every release:
//   * superblock version 0, 8-byte addresses and lengths, no user block;
//   * every group a symbol table: one version-1 B-tree node (type 0) over one symbol-table node
//     ("SNOD") whose names live in the group's local heap ("HEAP");
//   * every object a version-1 object header; datasets carry the fill-value (new form), datatype
//     (IEEE binary64, little-endian), dataspace (version 1) and contiguous data-layout (version 3)
//     messages, groups a symbol-table message.
// Raw data is appended as each dataset is written; the group structure and the superblock are
// written when the file is closed. Writing a path again replaces the dataset (dump_mode::overwrite;
// the earlier bytes stay in the file, unreferenced). Intermediate groups are created as needed.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "host_errors.h"
#include "sayram_gpu.h"
#include "sayram_h5.h"

namespace {

constexpr uint64_t kUndef = ~0ull;
constexpr int kInternalK = 16;  // group B-tree node: up to 2K children (libhdf5's default K)
constexpr int kMinLeafK = 4;    // symbol-table node: up to 2K entries (libhdf5's default K)
constexpr int kMaxLeafK = 65535;
constexpr size_t kSuperblock = 96;
constexpr size_t kEntry = 40;  // symbol-table entry

struct Node {
  bool group = true;
  // dataset
  std::vector<uint64_t> dims;
  uint64_t addr = kUndef, nbytes = 0;
  // group (std::map orders names byte-wise, as the B-tree's name comparison does)
  std::map<std::string, std::unique_ptr<Node>> kids;
  // filled in at close
  uint64_t ohdr = kUndef, btree = kUndef, heap = kUndef;
};

class Buf {  // little-endian serialisation
 public:
  std::vector<uint8_t> b;
  void u8(unsigned v) { b.push_back((uint8_t)v); }
  void u16(unsigned v) { u8(v & 0xff), u8((v >> 8) & 0xff); }
  void u32(uint32_t v) {
    for (int k = 0; k < 4; ++k) u8((v >> (8 * k)) & 0xff);
  }
  void u64(uint64_t v) {
    for (int k = 0; k < 8; ++k) u8((unsigned)((v >> (8 * k)) & 0xff));
  }
  void bytes(const void* p, size_t n) { b.insert(b.end(), (const uint8_t*)p, (const uint8_t*)p + n); }
  void zeros(size_t n) { b.insert(b.end(), n, 0); }
  void pad8() { zeros((8 - b.size() % 8) % 8); }
  size_t size() const { return b.size(); }
};

// one object-header message: type, body padded to 8 bytes, flags
struct Msg {
  unsigned type, flags;
  Buf body;
};

Buf object_header(std::vector<Msg>& msgs) {
  size_t total = 0;
  for (Msg& m : msgs) {
    m.body.pad8();
    total += 8 + m.body.size();
  }
  Buf h;
  h.u8(1);                      // version 1
  h.u8(0);                      // reserved
  h.u16((unsigned)msgs.size());  // number of messages
  h.u32(1);                     // object reference count
  h.u32((uint32_t)total);       // object header size
  h.zeros(4);                   // alignment of the first message
  for (Msg& m : msgs) {
    h.u16(m.type);
    h.u16((unsigned)m.body.size());
    h.u8(m.flags);
    h.zeros(3);
    h.bytes(m.body.b.data(), m.body.size());
  }
  return h;
}

}  // namespace

struct sayram_h5_s {
  FILE* fp = nullptr;
  uint64_t eof = 0;
  Node root;
  bool failed = false;

  int put(const Buf& x, uint64_t* at) {
    eof = (eof + 7) / 8 * 8;
    if (std::fseek(fp, (long)eof, SEEK_SET) != 0 || std::fwrite(x.b.data(), 1, x.size(), fp) != x.size())
      return sg::host_fail(SAYRAM_ERR_IO, "HDF5 output: write failed");
    if (at) *at = eof;
    eof += x.size();
    return SAYRAM_OK;
  }

  static size_t max_children(const Node& g) {
    size_t m = g.kids.size();
    for (const auto& kv : g.kids)
      if (kv.second->group) m = std::max(m, max_children(*kv.second));
    return m;
  }

  // children first, then the group's heap, symbol-table node, B-tree node and object header
  int emit(Node& g, int leaf_k) {
    for (auto& kv : g.kids) {
      Node& c = *kv.second;
      int rc = c.group ? emit(c, leaf_k) : emit_dataset(c);
      if (rc) return rc;
    }
    // local heap: "" at offset 0, the names (8-byte aligned), then one free block, as libhdf5 lays it out
    Buf data;
    data.zeros(8);
    std::vector<uint64_t> name_off;
    for (const auto& kv : g.kids) {
      name_off.push_back(data.size());
      data.bytes(kv.first.data(), kv.first.size());
      data.u8(0);
      data.pad8();
    }
    const uint64_t free_off = data.size();
    data.u64(1);   // next free block: none (libhdf5's end-of-list marker)
    data.u64(16);  // size of this free block
    Buf heap;
    heap.bytes("HEAP", 4);
    heap.u8(0);
    heap.zeros(3);
    heap.u64(data.size());
    heap.u64(free_off);
    const uint64_t heap_at = (eof + 7) / 8 * 8;
    heap.u64(heap_at + 32);  // the data segment follows the header
    heap.bytes(data.b.data(), data.size());
    int rc = put(heap, &g.heap);
    if (rc) return rc;
    // symbol-table node with every entry of the group, sorted by name
    uint64_t snod = kUndef;
    if (!g.kids.empty()) {
      Buf s;
      s.bytes("SNOD", 4);
      s.u8(1);
      s.u8(0);
      s.u16((unsigned)g.kids.size());
      size_t k = 0;
      for (const auto& kv : g.kids) {
        const Node& c = *kv.second;
        s.u64(name_off[k++]);
        s.u64(c.ohdr);
        s.u32(c.group ? 1 : 0);  // cache type 1: the group's B-tree and heap addresses follow
        s.u32(0);
        if (c.group) {
          s.u64(c.btree);
          s.u64(c.heap);
        } else {
          s.zeros(16);
        }
      }
      s.zeros(kEntry * (2 * (size_t)leaf_k - g.kids.size()));
      if ((rc = put(s, &snod))) return rc;
    }
    // B-tree root (level 0): keys "" and the last name, around the one symbol-table node
    Buf t;
    t.bytes("TREE", 4);
    t.u8(0);  // group node
    t.u8(0);  // level 0
    t.u16(g.kids.empty() ? 0 : 1);
    t.u64(kUndef);
    t.u64(kUndef);
    t.u64(0);
    if (!g.kids.empty()) {
      t.u64(snod);
      t.u64(name_off.back());
    }
    const size_t full = 24 + (2 * kInternalK + 1) * 8 + 2 * kInternalK * 8;
    t.zeros(full - t.size());
    if ((rc = put(t, &g.btree))) return rc;
    std::vector<Msg> msgs(1);
    msgs[0].type = 0x11;  // symbol table
    msgs[0].flags = 1;    // constant
    msgs[0].body.u64(g.btree);
    msgs[0].body.u64(g.heap);
    return put(object_header(msgs), &g.ohdr);
  }

  int emit_dataset(Node& d) {
    std::vector<Msg> msgs(4);
    // fill value (new form, version 1): allocation late, write if set, defined with size 0
    msgs[0].type = 0x5;
    msgs[0].flags = 1;
    msgs[0].body.u8(1);
    msgs[0].body.u8(2);
    msgs[0].body.u8(2);
    msgs[0].body.u8(1);
    msgs[0].body.u32(0);
    // datatype: version 1, floating point, little-endian, implied msb, sign at bit 63
    Buf& ty = msgs[1].body;
    msgs[1].type = 0x3;
    msgs[1].flags = 1;
    ty.u8(0x11);
    ty.u8(0x20);
    ty.u8(63);
    ty.u8(0);
    ty.u32(8);
    ty.u16(0);    // bit offset
    ty.u16(64);   // bit precision
    ty.u8(52);    // exponent location
    ty.u8(11);    // exponent size
    ty.u8(0);     // mantissa location
    ty.u8(52);    // mantissa size
    ty.u32(1023);  // exponent bias
    // dataspace: version 1, no maximum dimensions
    Buf& sp = msgs[2].body;
    msgs[2].type = 0x1;
    msgs[2].flags = 0;
    sp.u8(1);
    sp.u8((unsigned)d.dims.size());
    sp.u8(0);
    sp.zeros(5);
    for (uint64_t v : d.dims) sp.u64(v);
    // data layout: version 3, contiguous
    Buf& ly = msgs[3].body;
    msgs[3].type = 0x8;
    msgs[3].flags = 0;
    ly.u8(3);
    ly.u8(1);
    ly.u64(d.addr);
    ly.u64(d.nbytes);
    return put(object_header(msgs), &d.ohdr);
  }

  int finish() {
    const size_t mc = max_children(root);
    if (mc > 2 * (size_t)kMaxLeafK) return sg::host_fail(SAYRAM_ERR_ARG, "HDF5 output: too many entries in one group");
    const int leaf_k = (int)std::max<size_t>(kMinLeafK, (mc + 1) / 2);
    int rc = emit(root, leaf_k);
    if (rc) return rc;
    const uint64_t end = eof;
    Buf s;
    s.bytes("\x89HDF\r\n\x1a\n", 8);
    s.u8(0);  // superblock version
    s.u8(0);  // free-space storage version
    s.u8(0);  // root group symbol table entry version
    s.u8(0);
    s.u8(0);  // shared header message format version
    s.u8(8);  // size of offsets
    s.u8(8);  // size of lengths
    s.u8(0);
    s.u16((unsigned)leaf_k);
    s.u16(kInternalK);
    s.u32(0);  // file consistency flags
    s.u64(0);  // base address
    s.u64(kUndef);  // free-space info
    s.u64(end);     // end of file
    s.u64(kUndef);  // driver information block
    s.u64(0);       // root entry: link name offset
    s.u64(root.ohdr);
    s.u32(1);
    s.u32(0);
    s.u64(root.btree);
    s.u64(root.heap);
    if (s.size() != kSuperblock) return sg::host_fail(SAYRAM_ERR_IO, "HDF5 output: superblock size");
    if (std::fseek(fp, 0, SEEK_SET) != 0 || std::fwrite(s.b.data(), 1, s.size(), fp) != s.size())
      return sg::host_fail(SAYRAM_ERR_IO, "HDF5 output: write failed");
    return SAYRAM_OK;
  }
};

extern "C" {

int sayram_h5_create(const char* path, sayram_h5* out) {
  if (!path || !out) return sg::host_fail(SAYRAM_ERR_ARG, "sayram_h5_create: null argument");
  *out = nullptr;
  std::unique_ptr<sayram_h5_s> h(new (std::nothrow) sayram_h5_s);
  if (!h) return sg::host_fail(SAYRAM_ERR_OOM, "sayram_h5_create: out of host memory");
  h->fp = std::fopen(path, "w+b");  // HighFive::File::Overwrite truncates an existing file
  if (!h->fp) return sg::host_fail(SAYRAM_ERR_IO, std::string("cannot create ") + path);
  Buf z;
  z.zeros(kSuperblock);  // the superblock is written at close
  int rc = h->put(z, nullptr);
  if (rc) {
    std::fclose(h->fp);
    return rc;
  }
  *out = h.release();
  return SAYRAM_OK;
}

int sayram_h5_write(sayram_h5 h, const char* path, const double* data, int rank, const long long* dims) {
  if (!h || !path) return sg::host_fail(SAYRAM_ERR_ARG, "sayram_h5_write: null argument");
  if (h->failed) return sg::host_fail(SAYRAM_ERR_STATE, "sayram_h5_write: an earlier write failed");
  if (rank < 0 || rank > 32 || (rank > 0 && !dims))
    return sg::host_fail(SAYRAM_ERR_ARG, "sayram_h5_write: rank must be 0..32 with dims given");
  uint64_t n = 1;
  std::vector<uint64_t> d(rank);
  for (int k = 0; k < rank; ++k) {
    if (dims[k] < 0) return sg::host_fail(SAYRAM_ERR_ARG, "sayram_h5_write: negative dimension");
    d[k] = (uint64_t)dims[k];
    n *= d[k];
  }
  if (n > 0 && !data) return sg::host_fail(SAYRAM_ERR_ARG, "sayram_h5_write: null data");
  // split the path; every component but the last is a group
  std::vector<std::string> parts;
  std::string cur;
  for (const char* p = path;; ++p) {
    if (*p == '/' || *p == 0) {
      if (!cur.empty()) parts.push_back(cur);
      cur.clear();
      if (*p == 0) break;
    } else {
      cur.push_back(*p);
    }
  }
  if (parts.empty()) return sg::host_fail(SAYRAM_ERR_ARG, "sayram_h5_write: empty dataset name");
  for (const std::string& s : parts)
    if (s == "." || s == "..") return sg::host_fail(SAYRAM_ERR_ARG, "sayram_h5_write: '.' or '..' in a path");
  Node* g = &h->root;
  for (size_t k = 0; k + 1 < parts.size(); ++k) {
    auto it = g->kids.find(parts[k]);
    if (it == g->kids.end()) {
      it = g->kids.emplace(parts[k], std::unique_ptr<Node>(new Node)).first;
    } else if (!it->second->group) {
      return sg::host_fail(SAYRAM_ERR_ARG, std::string("sayram_h5_write: '") + parts[k] + "' is a dataset");
    }
    g = it->second.get();
  }
  auto it = g->kids.find(parts.back());
  if (it != g->kids.end() && it->second->group)
    return sg::host_fail(SAYRAM_ERR_ARG, std::string("sayram_h5_write: '") + path + "' is a group");
  std::unique_ptr<Node> ds(new Node);
  ds->group = false;
  ds->dims = d;
  ds->nbytes = n * 8;
  if (n > 0) {
    // FP64 little-endian: the host byte order on x86-64 and aarch64
    h->eof = (h->eof + 7) / 8 * 8;
    if (std::fseek(h->fp, (long)h->eof, SEEK_SET) != 0 || std::fwrite(data, 8, n, h->fp) != n) {
      h->failed = true;
      return sg::host_fail(SAYRAM_ERR_IO, "HDF5 output: write failed");
    }
    ds->addr = h->eof;
    h->eof += n * 8;
  }
  g->kids[parts.back()] = std::move(ds);
  return SAYRAM_OK;
}

int sayram_h5_close(sayram_h5 h) {
  if (!h) return sg::host_fail(SAYRAM_ERR_ARG, "sayram_h5_close: null handle");
  int rc = h->failed ? sg::host_fail(SAYRAM_ERR_STATE, "sayram_h5_close: an earlier write failed") : h->finish();
  if (std::fclose(h->fp) != 0 && rc == SAYRAM_OK) rc = sg::host_fail(SAYRAM_ERR_IO, "HDF5 output: close failed");
  delete h;
  return rc;
}

}  // extern "C"
