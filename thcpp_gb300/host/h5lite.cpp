// h5lite implementation (see h5lite.h).  Byte layouts follow the HDF5 File Format
// Specification 3.0: superblock (sec. II.A), v1 B-trees (III.A.1), symbol table nodes
// (III.B), local heaps (III.D), version-1 object headers (IV.A.1.a) and the dataspace,
// datatype, fill value, layout, filter pipeline, continuation and symbol table messages
// (IV.A.2).
#include "h5lite.h"

#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cstring>
#include <functional>
#include <tuple>

#if defined(__has_include)
#if __has_include(<zlib.h>)
#include <zlib.h>
#define H5LITE_ZLIB 1
#endif
#endif

namespace h5lite {

namespace {

constexpr uint64_t UNDEF = ~0ULL;
const uint8_t SIG[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};

uint64_t le(const uint8_t* p, int n)
{
  uint64_t v = 0;
  for (int i = n - 1; i >= 0; i--) v = (v << 8) | p[i];
  return v;
}

struct Msg {
  int type;
  std::vector<uint8_t> data;
};

struct Dtype {
  int cls = -1;     // 0 fixed, 1 float, 6 compound
  int size = 0;
  bool is_signed = true;
  bool big_endian = false;
  // compound complex: offsets of the two float members
  int re_off = -1, im_off = -1, part_size = 0;
};

struct Layout {
  int cls = -1;     // 0 compact, 1 contiguous, 2 chunked
  uint64_t addr = UNDEF, size = 0;
  std::vector<uint8_t> compact;
  std::vector<uint64_t> chunk;  // chunk dims (dataset rank)
};

struct Filter {
  int id;
  std::vector<uint32_t> vals;
};

struct DsetMeta {
  std::vector<uint64_t> dims;
  Dtype dt;
  Layout lay;
  std::vector<Filter> filters;
};

}  // namespace

struct Reader::Impl {
  int fd = -1;
  uint64_t base = 0;
  int so = 8, sl = 8;
  uint64_t root_oh = UNDEF;
  std::string path;

  std::vector<uint8_t> rd(uint64_t addr, uint64_t n) const
  {
    std::vector<uint8_t> b(n);
    uint64_t off = 0;
    while (off < n) {
      ssize_t r = pread(fd, b.data() + off, n - off, (off_t)(base + addr + off));
      if (r <= 0) throw Error("h5lite: read past end of " + path);
      off += (uint64_t)r;
    }
    return b;
  }

  std::vector<Msg> messages(uint64_t oh) const
  {
    auto pre = rd(oh, 16);
    if (pre[0] != 1) throw Error("h5lite: unsupported object header version in " + path);
    int nmsg = (int)le(&pre[2], 2);
    uint64_t hsize = le(&pre[8], 4);
    std::vector<Msg> out;
    std::vector<std::pair<uint64_t, uint64_t>> blocks{{oh + 16, hsize}};
    for (size_t bi = 0; bi < blocks.size() && (int)out.size() < nmsg; bi++) {
      auto blk = rd(blocks[bi].first, blocks[bi].second);
      size_t p = 0;
      while (p + 8 <= blk.size() && (int)out.size() < nmsg) {
        int type = (int)le(&blk[p], 2);
        size_t sz = (size_t)le(&blk[p + 2], 2);
        if (p + 8 + sz > blk.size()) break;
        Msg m{type, std::vector<uint8_t>(blk.begin() + p + 8, blk.begin() + p + 8 + sz)};
        if (type == 0x10) blocks.push_back({le(&m.data[0], so), le(&m.data[so], sl)});
        out.push_back(std::move(m));
        p += 8 + sz;
      }
    }
    return out;
  }

  // Members of the group whose object header is at `oh`: name -> object header address.
  std::map<std::string, uint64_t> members(uint64_t oh) const
  {
    std::map<std::string, uint64_t> out;
    for (auto& m : messages(oh)) {
      if (m.type != 0x11) continue;
      uint64_t bt = le(&m.data[0], so), heap = le(&m.data[so], so);
      auto hh = rd(heap, 8 + 2 * sl + so);
      if (memcmp(hh.data(), "HEAP", 4)) throw Error("h5lite: bad local heap");
      uint64_t dsize = le(&hh[8], sl), daddr = le(&hh[8 + 2 * sl], so);
      auto hdata = rd(daddr, dsize);
      std::function<void(uint64_t)> walk = [&](uint64_t node) {
        auto h = rd(node, 8 + 2 * so);
        if (!memcmp(h.data(), "SNOD", 4)) {
          int n = (int)le(&h[6], 2);
          size_t esz = 2 * so + 8 + 16;
          auto e = rd(node + 8, esz * n);
          for (int i = 0; i < n; i++) {
            uint64_t noff = le(&e[i * esz], so), addr = le(&e[i * esz + so], so);
            std::string name((const char*)&hdata[noff]);
            out[name] = addr;
          }
          return;
        }
        if (memcmp(h.data(), "TREE", 4)) throw Error("h5lite: bad B-tree node");
        int level = h[5];
        int used = (int)le(&h[6], 2);
        uint64_t hdr = 8 + 2 * so;
        auto kc = rd(node + hdr, (uint64_t)(used + 1) * sl + (uint64_t)used * so);
        for (int i = 0; i < used; i++) {
          uint64_t child = le(&kc[sl + (uint64_t)i * (sl + so)], so);
          (void)level;
          walk(child);
        }
      };
      walk(bt);
    }
    return out;
  }

  uint64_t lookup(const std::string& path) const
  {
    uint64_t oh = root_oh;
    size_t i = 0;
    while (i < path.size()) {
      while (i < path.size() && path[i] == '/') i++;
      if (i >= path.size()) break;
      size_t j = path.find('/', i);
      std::string part = path.substr(i, j == std::string::npos ? std::string::npos : j - i);
      auto mem = members(oh);
      auto it = mem.find(part);
      if (it == mem.end()) return UNDEF;
      oh = it->second;
      i = j == std::string::npos ? path.size() : j;
    }
    return oh;
  }

  static Dtype parse_dtype(const uint8_t* d, size_t n)
  {
    Dtype t;
    int ver = d[0] >> 4;
    t.cls = d[0] & 0x0f;
    t.size = (int)le(d + 4, 4);
    if (t.cls == 0) {
      t.big_endian = d[1] & 1;
      t.is_signed = (d[1] >> 3) & 1;
    } else if (t.cls == 1) {
      t.big_endian = d[1] & 1;
    } else if (t.cls == 6) {
      int nmemb = (int)le(d + 1, 2);
      size_t p = 8;
      for (int m = 0; m < nmemb && p < n; m++) {
        std::string name((const char*)d + p);
        size_t nl = name.size() + 1;
        if (ver < 3) nl = (nl + 7) / 8 * 8;
        p += nl;
        uint64_t off;
        if (ver < 3) {
          off = le(d + p, 4);
          p += 4 + 28;  // offset, then rank/perm/reserved/dims of the v1 member layout
        } else {
          int ob = t.size < 256 ? 1 : t.size < 65536 ? 2 : t.size < (1 << 24) ? 3 : 4;
          off = le(d + p, ob);
          p += ob;
        }
        Dtype mt = parse_dtype(d + p, n - p);
        size_t msz = member_bytes(d + p);
        p += msz;
        if (name == "r" || name == "real") { t.re_off = (int)off; t.part_size = mt.size; }
        if (name == "i" || name == "imag") t.im_off = (int)off;
        if (mt.cls != 1) t.re_off = -2;
      }
    }
    return t;
  }

  // Encoded size of a (non-compound) member datatype message.
  static size_t member_bytes(const uint8_t* d)
  {
    int cls = d[0] & 0x0f;
    if (cls == 0) return 8 + 4;
    if (cls == 1) return 8 + 12;
    throw Error("h5lite: nested datatype class not supported");
  }

  DsetMeta meta(const std::string& path) const
  {
    uint64_t oh = lookup(path);
    if (oh == UNDEF) throw Error("h5lite: no dataset " + path + " in " + this->path);
    DsetMeta dm;
    bool have_space = false;
    for (auto& m : messages(oh)) {
      const uint8_t* d = m.data.data();
      if (m.type == 0x1) {
        int ver = d[0], rank = d[1];
        size_t p = ver == 1 ? 8 : 4;
        dm.dims.clear();
        for (int r = 0; r < rank; r++) dm.dims.push_back(le(d + p + (size_t)r * sl, sl));
        have_space = true;
      } else if (m.type == 0x3) {
        dm.dt = parse_dtype(d, m.data.size());
      } else if (m.type == 0x8) {
        int ver = d[0];
        if (ver == 3) {
          dm.lay.cls = d[1];
          if (dm.lay.cls == 0) {
            size_t sz = le(d + 2, 2);
            dm.lay.compact.assign(d + 4, d + 4 + sz);
          } else if (dm.lay.cls == 1) {
            dm.lay.addr = le(d + 2, so);
            dm.lay.size = le(d + 2 + so, sl);
          } else if (dm.lay.cls == 2) {
            int r = d[2];
            dm.lay.addr = le(d + 3, so);
            for (int i = 0; i < r - 1; i++) dm.lay.chunk.push_back(le(d + 3 + so + 4 * i, 4));
          }
        } else if (ver == 1 || ver == 2) {
          int r = d[1];
          dm.lay.cls = d[2];
          size_t p = 8;
          if (dm.lay.cls != 0) {
            dm.lay.addr = le(d + p, so);
            p += so;
          }
          std::vector<uint64_t> cd;
          for (int i = 0; i < r; i++) cd.push_back(le(d + p + 4 * i, 4));
          if (dm.lay.cls == 2) dm.lay.chunk.assign(cd.begin(), cd.end() - 1);
        } else {
          throw Error("h5lite: layout message version not supported");
        }
      } else if (m.type == 0xB) {
        int ver = d[0], nf = d[1];
        size_t p = ver == 1 ? 8 : 2;
        for (int f = 0; f < nf; f++) {
          Filter fl;
          fl.id = (int)le(d + p, 2);
          size_t namelen = 0;
          if (ver == 1 || fl.id >= 256) namelen = le(d + p + 2, 2);
          size_t q = p + (ver == 1 || fl.id >= 256 ? 4 : 2);
          int nv = (int)le(d + q + 2, 2);
          q += 4;
          if (ver == 1) q += (namelen + 7) / 8 * 8;
          else q += namelen;
          for (int v = 0; v < nv; v++) fl.vals.push_back((uint32_t)le(d + q + 4 * v, 4));
          q += 4 * nv;
          if (ver == 1 && nv % 2) q += 4;
          dm.filters.push_back(fl);
          p = q;
        }
      }
    }
    if (!have_space || dm.dt.cls < 0 || dm.lay.cls < 0)
      throw Error("h5lite: " + path + " is not a dataset");
    return dm;
  }

  std::vector<uint8_t> raw(const DsetMeta& dm) const
  {
    uint64_t n = 1;
    for (auto x : dm.dims) n *= x;
    uint64_t bytes = n * dm.dt.size;
    if (dm.lay.cls == 0) return dm.lay.compact;
    if (dm.lay.cls == 1) {
      if (dm.lay.addr == UNDEF) return std::vector<uint8_t>(bytes, 0);
      return rd(dm.lay.addr, bytes);
    }
    // Chunked: walk the v1 B-tree of raw-data chunks.
    std::vector<uint8_t> out(bytes, 0);
    int rank = (int)dm.dims.size();
    uint64_t chunk_elems = 1;
    for (auto x : dm.lay.chunk) chunk_elems *= x;
    std::function<void(uint64_t)> walk = [&](uint64_t node) {
      auto h = rd(node, 8 + 2 * so);
      if (memcmp(h.data(), "TREE", 4)) throw Error("h5lite: bad chunk B-tree");
      int level = h[5], used = (int)le(&h[6], 2);
      size_t ksz = 8 + 8 * (size_t)(rank + 1);
      auto kc = rd(node + 8 + 2 * so, (uint64_t)(used + 1) * ksz + (uint64_t)used * so);
      for (int i = 0; i < used; i++) {
        const uint8_t* key = &kc[(size_t)i * (ksz + so)];
        uint64_t child = le(key + ksz, so);
        if (level > 0) {
          walk(child);
          continue;
        }
        uint32_t csize = (uint32_t)le(key, 4), mask = (uint32_t)le(key + 4, 4);
        std::vector<uint64_t> off(rank);
        for (int r = 0; r < rank; r++) off[r] = le(key + 8 + 8 * r, 8);
        auto data = rd(child, csize);
        for (int f = (int)dm.filters.size() - 1; f >= 0; f--) {
          if (mask & (1u << f)) continue;
          int id = dm.filters[f].id;
          if (id == 1) {
#ifdef H5LITE_ZLIB
            std::vector<uint8_t> dec(chunk_elems * dm.dt.size);
            uLongf dl = dec.size();
            if (uncompress(dec.data(), &dl, data.data(), data.size()) != Z_OK)
              throw Error("h5lite: deflate failed");
            dec.resize(dl);
            data.swap(dec);
#else
            throw Error("h5lite: deflate-compressed dataset but built without zlib");
#endif
          } else if (id == 2) {
            size_t es = dm.dt.size, ne = data.size() / es;
            std::vector<uint8_t> un(data.size());
            for (size_t b = 0; b < es; b++)
              for (size_t e = 0; e < ne; e++) un[e * es + b] = data[b * ne + e];
            data.swap(un);
          } else if (id == 3) {
            data.resize(data.size() - 4);
          } else {
            throw Error("h5lite: unsupported filter " + std::to_string(id));
          }
        }
        // Copy the chunk into place (clipped at the dataset edge).
        std::vector<uint64_t> idx(rank, 0);
        uint64_t ce = 0;
        while (true) {
          bool inside = true;
          uint64_t lin = 0;
          for (int r = 0; r < rank; r++) {
            uint64_t g = off[r] + idx[r];
            if (g >= dm.dims[r]) { inside = false; break; }
            lin = lin * dm.dims[r] + g;
          }
          if (inside && (ce + 1) * dm.dt.size <= data.size())
            memcpy(&out[lin * dm.dt.size], &data[ce * dm.dt.size], dm.dt.size);
          ce++;
          int r = rank - 1;
          while (r >= 0 && ++idx[r] == dm.lay.chunk[r]) idx[r--] = 0;
          if (r < 0) break;
        }
      }
    };
    if (dm.lay.addr != UNDEF) walk(dm.lay.addr);
    return out;
  }
};

Reader::Reader(const std::string& path) : p_(new Impl)
{
  p_->path = path;
  p_->fd = open(path.c_str(), O_RDONLY);
  if (p_->fd < 0) throw Error("h5lite: cannot open " + path);
  struct stat stt;
  fstat(p_->fd, &stt);
  uint64_t sb = UNDEF;
  for (uint64_t off = 0; off + 8 <= (uint64_t)stt.st_size; off = off ? off * 2 : 512) {
    uint8_t s[8];
    if (pread(p_->fd, s, 8, (off_t)off) == 8 && !memcmp(s, SIG, 8)) {
      sb = off;
      break;
    }
    if (off > (1ULL << 40)) break;
  }
  if (sb == UNDEF) throw Error("h5lite: " + path + " is not an HDF5 file");
  uint8_t h[256];
  ssize_t got = pread(p_->fd, h, sizeof h, (off_t)sb);
  if (got < 64) throw Error("h5lite: truncated superblock");
  int ver = h[8];
  if (ver > 1) throw Error("h5lite: superblock version " + std::to_string(ver) +
                           " not supported (write the file with libver='earliest')");
  p_->so = h[13];
  p_->sl = h[14];
  size_t p = 24 + (ver == 1 ? 4 : 0);
  p_->base = le(h + p, p_->so);
  p += 4 * p_->so;                              // base, free-space, EOF, driver info
  p_->root_oh = le(h + p + p_->so, p_->so);     // root symbol table entry: name off, header
  if (p_->base == 0 && sb != 0) p_->base = sb;
}

Reader::~Reader()
{
  if (p_ && p_->fd >= 0) close(p_->fd);
}

bool Reader::exists(const std::string& path) const { return p_->lookup(path) != UNDEF; }

bool Reader::is_group(const std::string& path) const
{
  uint64_t oh = p_->lookup(path);
  if (oh == UNDEF) return false;
  for (auto& m : p_->messages(oh))
    if (m.type == 0x11) return true;
  return false;
}

std::vector<std::string> Reader::list(const std::string& group) const
{
  uint64_t oh = p_->lookup(group);
  if (oh == UNDEF || !is_group(group)) throw Error("h5lite: no group " + group);
  std::vector<std::string> out;
  for (auto& kv : p_->members(oh)) out.push_back(kv.first);
  return out;
}

Info Reader::info(const std::string& path) const
{
  auto dm = p_->meta(path);
  Info i;
  i.dims = dm.dims;
  i.elem_size = dm.dt.size;
  i.kind = dm.dt.cls == 0 ? Kind::Int : dm.dt.cls == 1 ? Kind::Float
           : (dm.dt.cls == 6 && dm.dt.re_off >= 0 && dm.dt.im_off >= 0) ? Kind::Complex
                                                                        : Kind::Other;
  return i;
}

static double scalar(const uint8_t* p, const Dtype& t, int size, bool is_float)
{
  if (t.big_endian) throw Error("h5lite: big-endian data not supported");
  if (is_float) {
    if (size == 8) { double v; memcpy(&v, p, 8); return v; }
    if (size == 4) { float v; memcpy(&v, p, 4); return v; }
    throw Error("h5lite: unsupported float size");
  }
  uint64_t u = le(p, size);
  if (t.is_signed && size < 8 && (u >> (8 * size - 1)) & 1) u |= ~0ULL << (8 * size);
  return t.is_signed ? (double)(int64_t)u : (double)u;
}

std::vector<double> Reader::read_f64(const std::string& path, std::vector<uint64_t>* dims) const
{
  auto dm = p_->meta(path);
  if (dm.dt.cls != 0 && dm.dt.cls != 1) throw Error("h5lite: " + path + " is not real numeric");
  auto raw = p_->raw(dm);
  size_t n = raw.size() / dm.dt.size;
  std::vector<double> out(n);
  for (size_t i = 0; i < n; i++) out[i] = scalar(&raw[i * dm.dt.size], dm.dt, dm.dt.size, dm.dt.cls == 1);
  if (dims) *dims = dm.dims;
  return out;
}

std::vector<int> Reader::read_i32(const std::string& path, std::vector<uint64_t>* dims) const
{
  auto v = read_f64(path, dims);
  return std::vector<int>(v.begin(), v.end());
}

std::vector<double> Reader::read_c128(const std::string& path, std::vector<uint64_t>* dims) const
{
  auto dm = p_->meta(path);
  auto raw = p_->raw(dm);
  size_t n = raw.size() / dm.dt.size;
  std::vector<double> out(2 * n);
  if (dm.dt.cls == 6) {
    if (dm.dt.re_off < 0 || dm.dt.im_off < 0) throw Error("h5lite: " + path + " is not {r, i}");
    Dtype f;
    for (size_t i = 0; i < n; i++) {
      out[2 * i] = scalar(&raw[i * dm.dt.size + dm.dt.re_off], f, dm.dt.part_size, true);
      out[2 * i + 1] = scalar(&raw[i * dm.dt.size + dm.dt.im_off], f, dm.dt.part_size, true);
    }
  } else if (dm.dt.cls == 0 || dm.dt.cls == 1) {
    // Real data read as complex with zero imaginary part.
    for (size_t i = 0; i < n; i++) {
      out[2 * i] = scalar(&raw[i * dm.dt.size], dm.dt, dm.dt.size, dm.dt.cls == 1);
      out[2 * i + 1] = 0.0;
    }
  } else {
    throw Error("h5lite: " + path + " has an unsupported datatype");
  }
  if (dims) *dims = dm.dims;
  return out;
}

// ---------------------------------------------------------------------------- writer

struct Writer::Node {
  bool group = true;
  std::map<std::string, std::shared_ptr<Node>> kids;
  std::vector<uint64_t> dims;
  int kind = 0;            // 0 f64, 1 i32, 2 complex128 compound
  uint64_t addr = UNDEF, bytes = 0;
};

namespace {

struct Buf {
  std::vector<uint8_t> b;
  uint64_t base;
  void put(uint64_t v, int n) { for (int i = 0; i < n; i++) b.push_back((uint8_t)(v >> (8 * i))); }
  void bytes(const void* p, size_t n) { b.insert(b.end(), (const uint8_t*)p, (const uint8_t*)p + n); }
  void align8() { while (b.size() % 8) b.push_back(0); }
  uint64_t here() const { return base + b.size(); }
};

constexpr int LEAF_K = 32;      // symbol table nodes hold up to 2K = 64 entries
constexpr int INTERNAL_K = 16;

void message(Buf& o, int type, const std::vector<uint8_t>& data)
{
  size_t sz = (data.size() + 7) / 8 * 8;
  o.put(type, 2);
  o.put(sz, 2);
  o.put(0, 1);
  o.put(0, 3);
  o.bytes(data.data(), data.size());
  for (size_t i = data.size(); i < sz; i++) o.b.push_back(0);
}

uint64_t object_header(Buf& o, const std::vector<std::pair<int, std::vector<uint8_t>>>& msgs)
{
  o.align8();
  uint64_t at = o.here();
  size_t total = 0;
  for (auto& m : msgs) total += 8 + (m.second.size() + 7) / 8 * 8;
  o.put(1, 1);
  o.put(0, 1);
  o.put(msgs.size(), 2);
  o.put(1, 4);
  o.put(total, 4);
  o.put(0, 4);
  for (auto& m : msgs) message(o, m.first, m.second);
  return at;
}

std::vector<uint8_t> enc(std::initializer_list<std::pair<uint64_t, int>> f)
{
  std::vector<uint8_t> v;
  for (auto& x : f)
    for (int i = 0; i < x.second; i++) v.push_back((uint8_t)(x.first >> (8 * i)));
  return v;
}

}  // namespace

Writer::Writer(const std::string& path, bool truncate) : path_(path), root_(new Node)
{
  if (!truncate) {
    struct stat st;
    if (stat(path.c_str(), &st) == 0) {
      // Read every group and dataset, then rewrite the file and continue appending.
      std::vector<std::tuple<std::string, std::vector<uint64_t>, int, std::vector<uint8_t>>> items;
      std::vector<std::string> groups;
      {
        Reader r(path);
        std::function<void(const std::string&)> collect = [&](const std::string& g) {
          for (auto& name : r.list(g)) {
            std::string full = (g == "/" ? "" : g) + "/" + name;
            if (r.is_group(full)) {
              groups.push_back(full);
              collect(full);
              continue;
            }
            auto inf = r.info(full);
            std::vector<uint64_t> dims;
            std::vector<uint8_t> raw;
            int kind;
            if (inf.kind == Kind::Int) {
              auto v = r.read_i32(full, &dims);
              raw.assign((uint8_t*)v.data(), (uint8_t*)(v.data() + v.size()));
              kind = 1;
            } else if (inf.kind == Kind::Complex) {
              auto v = r.read_c128(full, &dims);
              raw.assign((uint8_t*)v.data(), (uint8_t*)(v.data() + v.size()));
              kind = 2;
            } else {
              auto v = r.read_f64(full, &dims);
              raw.assign((uint8_t*)v.data(), (uint8_t*)(v.data() + v.size()));
              kind = 0;
            }
            items.emplace_back(full, dims, kind, std::move(raw));
          }
        };
        collect("/");
      }
      int fd = open(path.c_str(), O_WRONLY | O_TRUNC);
      if (fd < 0) throw Error("h5lite: cannot rewrite " + path);
      ::close(fd);
      for (auto& g : groups) create_group(g);
      flush();
      for (auto& it : items)
        add(std::get<0>(it), std::get<1>(it), std::get<2>(it), std::get<3>(it).data(),
            std::get<3>(it).size());
      return;
    }
  }
  int fd = open(path.c_str(), O_WRONLY | O_CREAT | O_TRUNC, 0644);
  if (fd < 0) throw Error("h5lite: cannot create " + path);
  ::close(fd);
  flush();
}

void Writer::create_group(const std::string& path)
{
  auto n = root_;
  size_t i = 0;
  while (i < path.size()) {
    while (i < path.size() && path[i] == '/') i++;
    if (i >= path.size()) break;
    size_t j = path.find('/', i);
    std::string part = path.substr(i, j == std::string::npos ? std::string::npos : j - i);
    auto& k = n->kids[part];
    if (!k) k = std::make_shared<Node>();
    if (!k->group) throw Error("h5lite: " + part + " is a dataset");
    n = k;
    i = j == std::string::npos ? path.size() : j;
  }
}

void Writer::write_f64(const std::string& path, const std::vector<uint64_t>& dims, const double* d)
{
  uint64_t n = 1;
  for (auto x : dims) n *= x;
  add(path, dims, 0, d, n * 8);
}

void Writer::write_i32(const std::string& path, const std::vector<uint64_t>& dims, const int* d)
{
  uint64_t n = 1;
  for (auto x : dims) n *= x;
  add(path, dims, 1, d, n * 4);
}

void Writer::write_c128(const std::string& path, const std::vector<uint64_t>& dims, const double* d)
{
  uint64_t n = 1;
  for (auto x : dims) n *= x;
  add(path, dims, 2, d, n * 16);
}

void Writer::add(const std::string& path, const std::vector<uint64_t>& dims, int kind,
                 const void* data, size_t bytes)
{
  size_t slash = path.rfind('/');
  std::string parent = slash == std::string::npos || slash == 0 ? "/" : path.substr(0, slash);
  std::string name = path.substr(slash == std::string::npos ? 0 : slash + 1);
  create_group(parent);
  auto n = root_;
  if (parent != "/") {
    size_t i = 0;
    while (i < parent.size()) {
      while (i < parent.size() && parent[i] == '/') i++;
      if (i >= parent.size()) break;
      size_t j = parent.find('/', i);
      n = n->kids[parent.substr(i, j == std::string::npos ? std::string::npos : j - i)];
      i = j == std::string::npos ? parent.size() : j;
    }
  }
  if (n->kids.count(name)) throw Error("h5lite: " + path + " already exists");
  auto d = std::make_shared<Node>();
  d->group = false;
  d->dims = dims;
  d->kind = kind;
  d->bytes = bytes;
  // Append the raw data at the (8-byte aligned) end of file.
  uint64_t at = std::max<uint64_t>(eof_, 96);
  at = (at + 7) / 8 * 8;
  int fd = open(path_.c_str(), O_WRONLY);
  if (fd < 0) throw Error("h5lite: cannot write " + path_);
  size_t off = 0;
  while (off < bytes) {
    ssize_t w = pwrite(fd, (const uint8_t*)data + off, bytes - off, (off_t)(at + off));
    if (w <= 0) { ::close(fd); throw Error("h5lite: write failed"); }
    off += (size_t)w;
  }
  ::close(fd);
  d->addr = at;
  eof_ = at + bytes;
  n->kids[name] = d;
  flush();
}

void Writer::flush()
{
  uint64_t start = (std::max<uint64_t>(eof_, 96) + 7) / 8 * 8;
  Buf o{{}, start};
  struct GroupAddr { uint64_t oh, btree, heap; };
  std::function<GroupAddr(const Node&)> group = [&](const Node& g) -> GroupAddr {
    std::vector<std::pair<std::string, GroupAddr>> ent;
    for (auto& kv : g.kids) {
      if (kv.second->group) {
        ent.push_back({kv.first, group(*kv.second)});
      } else {
        const Node& d = *kv.second;
        int rank = (int)d.dims.size();
        std::vector<uint8_t> space = enc({{1, 1}, {(uint64_t)rank, 1}, {0, 1}, {0, 1}, {0, 4}});
        for (auto x : d.dims) for (int i = 0; i < 8; i++) space.push_back((uint8_t)(x >> (8 * i)));
        std::vector<uint8_t> dtype;
        std::vector<uint8_t> f64 = enc({{0x11, 1}, {0x20, 1}, {63, 1}, {0, 1}, {8, 4}, {0, 2},
                                        {64, 2}, {52, 1}, {11, 1}, {0, 1}, {52, 1}, {1023, 4}});
        if (d.kind == 0) {        // IEEE f64 little endian
          dtype = f64;
        } else if (d.kind == 1) { // signed 32-bit little endian
          dtype = enc({{0x10, 1}, {0x08, 1}, {0, 1}, {0, 1}, {4, 4}, {0, 2}, {32, 2}});
        } else {                  // compound {r, i} of f64, version-1 member encoding
          dtype = enc({{0x16, 1}, {2, 2}, {0, 1}, {16, 4}});
          const char* names[2] = {"r", "i"};
          for (int mbr = 0; mbr < 2; mbr++) {
            std::vector<uint8_t> nm(8, 0);
            nm[0] = (uint8_t)names[mbr][0];
            dtype.insert(dtype.end(), nm.begin(), nm.end());
            auto off = enc({{(uint64_t)(8 * mbr), 4}});
            dtype.insert(dtype.end(), off.begin(), off.end());
            dtype.insert(dtype.end(), 28, 0);  // dimensionality, permutation, dims: scalar
            dtype.insert(dtype.end(), f64.begin(), f64.end());
          }
        }
        std::vector<uint8_t> fill = enc({{2, 1}, {1, 1}, {2, 1}, {0, 1}});
        std::vector<uint8_t> layout = enc({{3, 1}, {1, 1}, {d.addr, 8}, {d.bytes, 8}});
        uint64_t oh = object_header(o, {{1, space}, {3, dtype}, {5, fill}, {8, layout}});
        ent.push_back({kv.first, {oh, UNDEF, UNDEF}});
      }
    }
    if (ent.size() > 2 * LEAF_K) throw Error("h5lite: too many members in one group");
    // Local heap with the names ("" at offset 0).
    std::vector<uint8_t> names(8, 0);
    std::vector<uint64_t> noff;
    for (auto& e : ent) {
      noff.push_back(names.size());
      names.insert(names.end(), e.first.begin(), e.first.end());
      names.push_back(0);
      while (names.size() % 8) names.push_back(0);
    }
    o.align8();
    uint64_t heap_data = o.here();
    o.bytes(names.data(), names.size());
    o.align8();
    uint64_t heap = o.here();
    o.bytes("HEAP", 4);
    o.put(0, 1);
    o.put(0, 3);
    o.put(names.size(), 8);
    o.put(UNDEF, 8);
    o.put(heap_data, 8);
    // Symbol table node (full 2K capacity).
    o.align8();
    uint64_t snod = o.here();
    o.bytes("SNOD", 4);
    o.put(1, 1);
    o.put(0, 1);
    o.put(ent.size(), 2);
    for (int i = 0; i < 2 * LEAF_K; i++) {
      if (i < (int)ent.size()) {
        const GroupAddr& a = ent[i].second;
        o.put(noff[i], 8);
        o.put(a.oh, 8);
        bool isg = a.btree != UNDEF;
        o.put(isg ? 1 : 0, 4);
        o.put(0, 4);
        o.put(isg ? a.btree : 0, 8);
        o.put(isg ? a.heap : 0, 8);
      } else {
        for (int b = 0; b < 40; b++) o.b.push_back(0);
      }
    }
    // Group B-tree: one leaf pointing at the symbol table node.
    o.align8();
    uint64_t bt = o.here();
    o.bytes("TREE", 4);
    o.put(0, 1);
    o.put(0, 1);
    o.put(ent.empty() ? 0 : 1, 2);
    o.put(UNDEF, 8);
    o.put(UNDEF, 8);
    for (int i = 0; i < 2 * INTERNAL_K + 1; i++) {
      uint64_t key = 0;
      if (i == 1 && !ent.empty()) key = noff.back();
      o.put(key, 8);
      if (i < 2 * INTERNAL_K) o.put(i == 0 && !ent.empty() ? snod : 0, 8);
    }
    uint64_t oh = object_header(o, {{0x11, enc({{bt, 8}, {heap, 8}})}});
    return {oh, bt, heap};
  };
  GroupAddr root = group(*root_);
  uint64_t eof = o.here();
  Buf sb{{}, 0};
  sb.bytes(SIG, 8);
  sb.put(0, 1);  // superblock version
  sb.put(0, 1);  // free-space version
  sb.put(0, 1);  // root group symbol table entry version
  sb.put(0, 1);
  sb.put(0, 1);  // shared header message format version
  sb.put(8, 1);  // size of offsets
  sb.put(8, 1);  // size of lengths
  sb.put(0, 1);
  sb.put(LEAF_K, 2);
  sb.put(INTERNAL_K, 2);
  sb.put(0, 4);
  sb.put(0, 8);      // base address
  sb.put(UNDEF, 8);  // free-space info
  sb.put(eof, 8);    // end of file
  sb.put(UNDEF, 8);  // driver information block
  sb.put(0, 8);      // root entry: link name offset
  sb.put(root.oh, 8);
  sb.put(1, 4);
  sb.put(0, 4);
  sb.put(root.btree, 8);
  sb.put(root.heap, 8);
  int fd = open(path_.c_str(), O_WRONLY);
  if (fd < 0) throw Error("h5lite: cannot write " + path_);
  bool ok = pwrite(fd, o.b.data(), o.b.size(), (off_t)start) == (ssize_t)o.b.size() &&
            pwrite(fd, sb.b.data(), sb.b.size(), 0) == (ssize_t)sb.b.size();
  if (ftruncate(fd, (off_t)eof) != 0) ok = false;
  ::close(fd);
  if (!ok) throw Error("h5lite: write failed for " + path_);
  eof_ = eof;
}

}  // namespace h5lite
