// lx_hdf5.cpp -- minimal HDF5 writer and reader for the reference's snapshot layout.
//
// The reference writes one file per field, one dataset per snapshot named "t=<step>"
// (writeHDF5 formats the step as a C++ stream double, fileio.cc:186-187), native double,
// contiguous, dataspace = global staggered extents (fileio.cc:143-157).  There is no libhdf5
// on this machine or the GPU hosts, so this file writes that subset of the HDF5 file format
// (public specification) directly:
//   superblock version 0, 8-byte offsets and lengths;
//   root group = version-1 object header with a Symbol Table message -> version-1 group
//   B-tree (one leaf) -> one symbol-table node (capacity sized to the dataset count, names
//   sorted) + a local heap of names;
//   datasets = version-1 object headers with Dataspace (v1), Datatype (IEEE double LE),
//   Fill Value (v2, undefined) and Layout (v3, contiguous) messages.
// Raw data is appended while the run goes; all metadata is written at close, and the
// superblock is rewritten last.  The reader parses the same subset (plus multi-level group
// B-trees, object-header continuations and 32-bit floats), which is what material files
// written by h5py with default settings use.
#include "lx_hdf5.h"

#include <algorithm>
#include <cerrno>
#include <cstdint>
#include <cstring>
#include <sstream>

#include "luxum.h"

namespace lx {

namespace {

constexpr uint64_t kUndef = ~0ull;
constexpr uint64_t kHeapFreeNull = 1;  // "no free block" value of the local heap's free list

void put16(std::vector<uint8_t>& b, uint16_t v) {
  for (int i = 0; i < 2; i++) b.push_back((uint8_t)(v >> (8 * i)));
}
void put32(std::vector<uint8_t>& b, uint32_t v) {
  for (int i = 0; i < 4; i++) b.push_back((uint8_t)(v >> (8 * i)));
}
void put64(std::vector<uint8_t>& b, uint64_t v) {
  for (int i = 0; i < 8; i++) b.push_back((uint8_t)(v >> (8 * i)));
}
void pad8(std::vector<uint8_t>& b) {
  while (b.size() % 8) b.push_back(0);
}

// One version-1 object header message (type, data padded to 8 bytes).
void message(std::vector<uint8_t>& hdr, uint16_t type, const std::vector<uint8_t>& data, uint8_t flags = 0) {
  std::vector<uint8_t> d = data;
  pad8(d);
  put16(hdr, type);
  put16(hdr, (uint16_t)d.size());
  hdr.push_back(flags);
  hdr.push_back(0);
  hdr.push_back(0);
  hdr.push_back(0);
  hdr.insert(hdr.end(), d.begin(), d.end());
}

std::vector<uint8_t> object_header(const std::vector<uint8_t>& msgs, uint16_t nmsgs) {
  std::vector<uint8_t> h;
  h.push_back(1);  // version
  h.push_back(0);
  put16(h, nmsgs);
  put32(h, 1);  // reference count
  put32(h, (uint32_t)msgs.size());
  put32(h, 0);  // alignment of the first message to 8 bytes
  h.insert(h.end(), msgs.begin(), msgs.end());
  return h;
}

// "t=" << double t, as std::ostringstream prints it (default precision 6, %g style)
std::string dataset_name(int t) {
  std::ostringstream os;
  os << "t=" << (double)t;
  return os.str();
}

}  // namespace

Hdf5Writer::~Hdf5Writer() { close(); }

std::string Hdf5Writer::failed(const char* what) const {
  return std::string(what) + " failed on " + path_ + ": " + std::strerror(errno);
}

std::string Hdf5Writer::open(const char* path, const int ext[3]) {
  f_ = std::fopen(path, "wb+");
  if (!f_) return std::string("cannot create ") + path + ": " + std::strerror(errno);
  path_ = path;
  for (int a = 0; a < 3; a++) ext_[a] = ext[a];
  std::vector<uint8_t> zeros(96, 0);
  if (std::fwrite(zeros.data(), 1, zeros.size(), f_) != zeros.size()) return failed("write");
  eof_ = 96;
  return "";
}

std::string Hdf5Writer::write(int t, const double* data) { return write_named(dataset_name(t), data); }

std::string Hdf5Writer::write_named(const std::string& name, const double* data, const int* ext) {
  if (!f_) return "HDF5 file is not open";
  if (!ext) ext = ext_;
  const uint64_t n = (uint64_t)ext[0] * ext[1] * ext[2];
  Entry e;
  e.name = name;
  for (int a = 0; a < 3; a++) e.ext[a] = ext[a];
  e.addr = eof_;
  e.bytes = n * 8;
  if (std::fseek(f_, (long)eof_, SEEK_SET) != 0) return failed("seek");
  // native double is little-endian IEEE on every host this builds for
  if (n && std::fwrite(data, 8, n, f_) != n) return failed("write");
  eof_ += e.bytes;
  while (eof_ % 8) {
    std::fputc(0, f_);
    eof_++;
  }
  for (auto& old : entries_)
    if (old.name == e.name) return "dataset " + e.name + " written twice";
  entries_.push_back(e);
  return "";
}

std::string Hdf5Writer::close() {
  if (!f_) return "";
  std::vector<uint8_t> meta;
  const uint64_t base = eof_;
  auto here = [&]() { return base + meta.size(); };
  // local heap: "" at offset 0, then the names
  std::vector<Entry> ents = entries_;
  std::sort(ents.begin(), ents.end(), [](const Entry& a, const Entry& b) { return std::strcmp(a.name.c_str(), b.name.c_str()) < 0; });
  std::vector<uint8_t> heap_data(8, 0);
  std::vector<uint64_t> name_off;
  for (auto& e : ents) {
    name_off.push_back(heap_data.size());
    heap_data.insert(heap_data.end(), e.name.begin(), e.name.end());
    heap_data.push_back(0);
    pad8(heap_data);
  }
  // dataset object headers
  std::vector<uint64_t> obj_addr;
  for (auto& e : ents) {
    std::vector<uint8_t> msgs, d;
    d = {1, 3, 0, 0, 0, 0, 0, 0};  // dataspace v1, rank 3, no max dims
    for (int a = 0; a < 3; a++) put64(d, (uint64_t)e.ext[a]);
    message(msgs, 0x0001, d);
    d = {0x11, 0x20, 63, 0};  // datatype v1 class float: LE, implied msb, sign bit 63
    put32(d, 8);
    put16(d, 0);
    put16(d, 64);
    d.push_back(52);
    d.push_back(11);
    d.push_back(0);
    d.push_back(52);
    put32(d, 1023);
    message(msgs, 0x0003, d, 1);
    d = {2, 2, 2, 0};  // fill value v2: late allocation, write if set, undefined
    message(msgs, 0x0005, d, 1);
    d = {3, 1};  // layout v3 contiguous
    put64(d, e.addr);
    put64(d, e.bytes);
    message(msgs, 0x0008, d);
    obj_addr.push_back(here());
    auto oh = object_header(msgs, 4);
    meta.insert(meta.end(), oh.begin(), oh.end());
    pad8(meta);
  }
  // heap header + data
  const uint64_t heap_addr = here();
  std::vector<uint8_t> hh = {'H', 'E', 'A', 'P', 0, 0, 0, 0};
  put64(hh, heap_data.size());
  put64(hh, kHeapFreeNull);
  put64(hh, heap_addr + 32);
  meta.insert(meta.end(), hh.begin(), hh.end());
  meta.insert(meta.end(), heap_data.begin(), heap_data.end());
  pad8(meta);
  // symbol table node (capacity 2K entries)
  const uint32_t leafK = (uint32_t)std::max<size_t>(4, (ents.size() + 1) / 2);
  const uint32_t intK = 16;
  const uint64_t snod_addr = here();
  std::vector<uint8_t> sn = {'S', 'N', 'O', 'D', 1, 0};
  put16(sn, (uint16_t)ents.size());
  for (size_t q = 0; q < 2 * (size_t)leafK; q++) {
    if (q < ents.size()) {
      put64(sn, name_off[q]);
      put64(sn, obj_addr[q]);
    } else {
      put64(sn, 0);
      put64(sn, 0);
    }
    put32(sn, 0);
    put32(sn, 0);
    for (int z = 0; z < 16; z++) sn.push_back(0);
  }
  meta.insert(meta.end(), sn.begin(), sn.end());
  pad8(meta);
  // group B-tree: one leaf pointing at the symbol table node; keys "" and the last name
  const uint64_t btree_addr = here();
  std::vector<uint8_t> bt = {'T', 'R', 'E', 'E', 0, 0};
  put16(bt, ents.empty() ? 0 : 1);
  put64(bt, kUndef);
  put64(bt, kUndef);
  put64(bt, 0);
  if (!ents.empty()) {
    put64(bt, snod_addr);
    put64(bt, name_off.back());
  }
  const size_t bt_size = 24 + (2 * intK + 1) * 8 + 2 * intK * 8;
  while (bt.size() < bt_size) bt.push_back(0);
  meta.insert(meta.end(), bt.begin(), bt.end());
  pad8(meta);
  // root group object header
  const uint64_t root_addr = here();
  std::vector<uint8_t> msgs, d;
  put64(d, btree_addr);
  put64(d, heap_addr);
  message(msgs, 0x0011, d);
  auto oh = object_header(msgs, 1);
  meta.insert(meta.end(), oh.begin(), oh.end());
  pad8(meta);
  const uint64_t eof = here();
  // superblock version 0
  std::vector<uint8_t> sb = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n', 0, 0, 0, 0, 0, 8, 8, 0};
  put16(sb, (uint16_t)leafK);
  put16(sb, (uint16_t)intK);
  put32(sb, 0);
  put64(sb, 0);
  put64(sb, kUndef);
  put64(sb, eof);
  put64(sb, kUndef);
  put64(sb, 0);  // root symbol table entry: name offset
  put64(sb, root_addr);
  put32(sb, 1);  // cache type 1: scratch-pad holds B-tree and heap addresses
  put32(sb, 0);
  put64(sb, btree_addr);
  put64(sb, heap_addr);
  std::string err;
  if (std::fseek(f_, (long)base, SEEK_SET) != 0 || std::fwrite(meta.data(), 1, meta.size(), f_) != meta.size())
    err = failed("metadata write");
  if (err.empty() && (std::fseek(f_, 0, SEEK_SET) != 0 || std::fwrite(sb.data(), 1, sb.size(), f_) != sb.size()))
    err = failed("superblock write");
  if (std::fclose(f_) != 0 && err.empty()) err = failed("close");
  f_ = nullptr;
  return err;
}

// ------------------------------------------------------------------ reader

namespace {

struct Reader {
  std::FILE* f = nullptr;
  std::string err;
  int leafK = 4;
  bool read(uint64_t addr, void* dst, size_t n) {
    if (std::fseek(f, (long)addr, SEEK_SET) != 0 || std::fread(dst, 1, n, f) != n) {
      err = "truncated file";
      return false;
    }
    return true;
  }
  static uint64_t le(const uint8_t* p, int n) {
    uint64_t v = 0;
    for (int i = n - 1; i >= 0; i--) v = (v << 8) | p[i];
    return v;
  }
  bool heap_name(uint64_t heap, uint64_t off, std::string& name) {
    uint8_t h[32];
    if (!read(heap, h, 32) || std::memcmp(h, "HEAP", 4) != 0) {
      if (err.empty()) err = "bad local heap";
      return false;
    }
    uint64_t data = le(h + 24, 8);
    name.clear();
    for (uint64_t q = 0;; q++) {
      uint8_t ch;
      if (!read(data + off + q, &ch, 1)) return false;
      if (!ch) break;
      name += (char)ch;
      if (q > 4096) { err = "bad name"; return false; }
    }
    return true;
  }
  // walks a group B-tree for `want`; returns the object header address or kUndef
  uint64_t find(uint64_t btree, uint64_t heap, const std::string& want, int depth = 0) {
    if (depth > 16) { err = "group tree too deep"; return kUndef; }
    uint8_t h[24];
    if (!read(btree, h, 24) || std::memcmp(h, "TREE", 4) != 0) { if (err.empty()) err = "bad group B-tree"; return kUndef; }
    const int level = h[5];
    const int used = (int)le(h + 6, 2);
    std::vector<uint8_t> body((size_t)(2 * used + 1) * 8);
    if (!read(btree + 24, body.data(), body.size())) return kUndef;
    for (int c = 0; c < used; c++) {
      uint64_t child = le(body.data() + (2 * c + 1) * 8, 8);
      if (level > 0) {
        uint64_t r = find(child, heap, want, depth + 1);
        if (r != kUndef || !err.empty()) return r;
        continue;
      }
      uint8_t sh[8];
      if (!read(child, sh, 8) || std::memcmp(sh, "SNOD", 4) != 0) { if (err.empty()) err = "bad symbol table node"; return kUndef; }
      const int nsym = (int)le(sh + 6, 2);
      std::vector<uint8_t> ent((size_t)nsym * 40);
      if (!read(child + 8, ent.data(), ent.size())) return kUndef;
      for (int e = 0; e < nsym; e++) {
        std::string name;
        if (!heap_name(heap, le(ent.data() + e * 40, 8), name)) return kUndef;
        if (name == want) return le(ent.data() + e * 40 + 8, 8);
      }
    }
    return kUndef;
  }
  // collects the messages of a version-1 object header (following continuations)
  bool messages(uint64_t addr, std::vector<std::pair<int, std::vector<uint8_t>>>& out) {
    uint8_t h[16];
    if (!read(addr, h, 16)) return false;
    if (h[0] != 1) { err = "only version-1 object headers are supported"; return false; }
    int nmsg = (int)le(h + 2, 2);
    std::vector<std::pair<uint64_t, uint64_t>> chunks = {{addr + 16, le(h + 8, 4)}};
    for (size_t ci = 0; ci < chunks.size() && (int)out.size() < nmsg; ci++) {
      std::vector<uint8_t> c(chunks[ci].second);
      if (!read(chunks[ci].first, c.data(), c.size())) return false;
      size_t p = 0;
      while (p + 8 <= c.size() && (int)out.size() < nmsg) {
        int type = (int)le(&c[p], 2);
        size_t sz = (size_t)le(&c[p + 2], 2);
        if (p + 8 + sz > c.size()) { err = "bad object header message"; return false; }
        std::vector<uint8_t> d(c.begin() + p + 8, c.begin() + p + 8 + sz);
        if (type == 0x0010 && sz >= 16) chunks.push_back({le(d.data(), 8), le(d.data() + 8, 8)});
        out.push_back({type, d});
        p += 8 + sz;
      }
    }
    return true;
  }
};

}  // namespace

std::string hdf5_read(const char* path, const char* dataset, std::vector<double>& data, int shape[3]) {
  Reader r;
  r.f = std::fopen(path, "rb");
  if (!r.f) return std::string("cannot open ") + path;
  struct Closer {
    std::FILE* f;
    ~Closer() { std::fclose(f); }
  } closer{r.f};
  uint8_t sb[96];
  if (!r.read(0, sb, 96)) return r.err;
  const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
  if (std::memcmp(sb, sig, 8) != 0) return std::string(path) + " is not an HDF5 file";
  if (sb[8] != 0 && sb[8] != 1) return "only superblock versions 0 and 1 are supported";
  if (sb[13] != 8 || sb[14] != 8) return "only 8-byte offsets and lengths are supported";
  const size_t ent = sb[8] == 0 ? 56 : 60;  // v1 adds 4 bytes (indexed storage K + reserved)
  uint64_t btree = Reader::le(sb + ent + 24, 8), heap = Reader::le(sb + ent + 32, 8);
  if (Reader::le(sb + ent + 16, 4) != 1) {  // no cached scratch-pad: read the root's Symbol Table message
    std::vector<std::pair<int, std::vector<uint8_t>>> rm;
    if (!r.messages(Reader::le(sb + ent + 8, 8), rm)) return r.err;
    btree = kUndef;
    for (auto& m : rm)
      if (m.first == 0x0011 && m.second.size() >= 16) {
        btree = Reader::le(m.second.data(), 8);
        heap = Reader::le(m.second.data() + 8, 8);
      }
    if (btree == kUndef) return "root group has no symbol table (only old-style groups are supported)";
  }
  uint64_t obj = r.find(btree, heap, dataset);
  if (!r.err.empty()) return r.err;
  if (obj == kUndef) return std::string("dataset \"") + dataset + "\" not found in " + path;
  std::vector<std::pair<int, std::vector<uint8_t>>> msgs;
  if (!r.messages(obj, msgs)) return r.err;
  int rank = -1, elsize = 0, cls = -1;
  uint64_t dims[3] = {1, 1, 1}, addr = kUndef, bytes = 0;
  bool big = false;
  for (auto& m : msgs) {
    const auto& d = m.second;
    if (m.first == 0x0001 && d.size() >= 8) {
      rank = d[1];
      size_t off = d[0] == 1 ? 8 : 4;
      if (rank > 3) return "datasets of rank > 3 are not supported";
      for (int a = 0; a < rank; a++) dims[3 - rank + a] = Reader::le(d.data() + off + 8 * a, 8);
    } else if (m.first == 0x0003 && d.size() >= 8) {
      cls = d[0] & 0x0f;
      big = (d[1] & 1) != 0;
      elsize = (int)Reader::le(d.data() + 4, 4);
    } else if (m.first == 0x0008 && d.size() >= 2) {
      if (d[0] != 3 || d[1] != 1) return "only contiguous (layout v3) datasets are supported";
      addr = Reader::le(d.data() + 2, 8);
      bytes = Reader::le(d.data() + 10, 8);
    } else if (m.first == 0x000B) {
      return "filtered (compressed) datasets are not supported";
    }
  }
  if (rank < 0 || cls != 1 || (elsize != 8 && elsize != 4) || big) return "dataset must be little-endian float32/float64";
  const uint64_t n = dims[0] * dims[1] * dims[2];
  if (addr == kUndef || bytes < n * (uint64_t)elsize) return "dataset storage missing or short";
  data.resize(n);
  if (elsize == 8) {
    if (!r.read(addr, data.data(), n * 8)) return r.err;
  } else {
    std::vector<float> tmp(n);
    if (!r.read(addr, tmp.data(), n * 4)) return r.err;
    for (uint64_t q = 0; q < n; q++) data[q] = tmp[q];
  }
  for (int a = 0; a < 3; a++) shape[a] = (int)dims[a];
  return "";
}

lx_status set_thread_error(const char* msg, lx_status st);

}  // namespace lx

extern "C" LX_API lx_status lx_hdf5_write(const char* path, int ndatasets, const char* const* names,
                                          const double* const* data, const int shape[3]) {
  if (!path || ndatasets < 0 || (ndatasets && (!names || !data)) || !shape)
    return lx::set_thread_error("null argument", LX_ERR_INVALID);
  lx::Hdf5Writer w;
  std::string err = w.open(path, shape);
  for (int q = 0; q < ndatasets && err.empty(); q++) err = w.write_named(names[q], data[q]);
  std::string cerr = w.close();
  if (err.empty()) err = cerr;
  if (!err.empty()) return lx::set_thread_error(err.c_str(), LX_ERR_IO);
  return LX_OK;
}

extern "C" LX_API lx_status lx_hdf5_read(const char* path, const char* dataset, double* out, size_t n, int shape[3]) {
  if (!path || !dataset || !shape) return lx::set_thread_error("null argument", LX_ERR_INVALID);
  std::vector<double> data;
  std::string err = lx::hdf5_read(path, dataset, data, shape);
  if (!err.empty()) return lx::set_thread_error(err.c_str(), LX_ERR_IO);
  if (out) {
    if (n != data.size()) return lx::set_thread_error("buffer size does not match the dataset", LX_ERR_INVALID);
    std::memcpy(out, data.data(), n * sizeof(double));
  }
  return LX_OK;
}
