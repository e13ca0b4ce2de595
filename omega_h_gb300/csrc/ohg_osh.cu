// .osh files: a device-resident mesh written to, and read from, one part of
// the reference's binary mesh format (src/Omega_h_file.cpp).  The format is
// the reference's own, so the layout below is fixed by it:
//   magic a1 1a, I8 compressed, meta (I8 family, I8 dim, I32 comm size, I32
//   comm rank, I8 parting, I32 ghost layers, I8 hints), LO nverts, the down
//   adjacencies (and their codes from faces up), per dimension the tags
//   (name, I8 ncomps, I8 type, array), the class sets, I8 has_parents;
// every array is LO size then the raw bytes or I64 compressed bytes and a
// zlib stream (compress2 at Z_BEST_SPEED, as the reference writes them).
// The arrays move between host and device in one copy each; zlib, when
// asked for, runs on the host (loaded at run time, so the library does not
// link against it).
#include <dlfcn.h>
#include <sys/stat.h>

#include <algorithm>
#include <cstring>
#include <fstream>
#include <sstream>

#include "ohg_mesh.cuh"

namespace ohg {

namespace {

constexpr unsigned char kMagic[2] = {0xa1, 0x1a};
constexpr int kLatestVersion = 9;
enum TagType { T_I8 = 0, T_I32 = 2, T_I64 = 3, T_F64 = 5 };

int type_size(int t) {
  switch (t) {
    case T_I8:
      return 1;
    case T_I32:
      return 4;
    case T_I64:
    case T_F64:
      return 8;
  }
  throw Error(1, ".osh: unknown tag type " + std::to_string(t));
}

// zlib entry points, resolved once from the system's libz
struct Zlib {
  typedef int (*Compress2)(unsigned char*, unsigned long*, const unsigned char*, unsigned long,
                           int);
  typedef unsigned long (*Bound)(unsigned long);
  typedef int (*Uncompress)(unsigned char*, unsigned long*, const unsigned char*, unsigned long);
  Compress2 compress2 = nullptr;
  Bound bound = nullptr;
  Uncompress uncompress = nullptr;
  Zlib() {
    void* h = dlopen("libz.so.1", RTLD_NOW | RTLD_LOCAL);
    if (!h) h = dlopen("libz.so", RTLD_NOW | RTLD_LOCAL);
    if (!h) return;
    compress2 = reinterpret_cast<Compress2>(dlsym(h, "compress2"));
    bound = reinterpret_cast<Bound>(dlsym(h, "compressBound"));
    uncompress = reinterpret_cast<Uncompress>(dlsym(h, "uncompress"));
    if (!compress2 || !bound || !uncompress) compress2 = nullptr;
  }
  bool ok() const { return compress2 != nullptr; }
};
const Zlib& zlib() {
  static Zlib z;
  return z;
}

class Out {
 public:
  explicit Out(bool compress) : compress_(compress) {}
  template <class T>
  void val(T v) {
    const char* p = reinterpret_cast<const char*>(&v);
    buf_.insert(buf_.end(), p, p + sizeof(T));
  }
  void bytes(const void* p, size_t n) {
    const char* c = static_cast<const char*>(p);
    buf_.insert(buf_.end(), c, c + n);
  }
  void str(const std::string& s) {
    val<std::int32_t>(std::int32_t(s.size()));
    bytes(s.data(), s.size());
  }
  // one array: LO size, then raw or zlib bytes
  void array(const void* host, LO n, int esize) {
    val<LO>(n);
    size_t nb = size_t(n) * size_t(esize);
    if (!compress_) {
      bytes(host, nb);
      return;
    }
    const Zlib& z = zlib();
    unsigned long cap = z.bound(nb);
    std::vector<unsigned char> c(cap ? cap : 1);
    unsigned long got = cap;
    int rc = z.compress2(c.data(), &got, static_cast<const unsigned char*>(host), nb, 1);
    if (rc != 0) throw Error(1, ".osh: zlib compress2 failed");
    val<std::int64_t>(std::int64_t(got));
    bytes(c.data(), got);
  }
  template <class T>
  void device_array(const Arr<T>& a) {
    std::vector<T> h = to_host(a);
    array(h.data(), a.size(), int(sizeof(T)));
  }
  const std::vector<char>& buf() const { return buf_; }

 private:
  bool compress_;
  std::vector<char> buf_;
};

class In {
 public:
  explicit In(std::vector<char> b) : b_(std::move(b)) {}
  template <class T>
  T val() {
    T v;
    need(sizeof(T));
    std::memcpy(&v, b_.data() + p_, sizeof(T));
    p_ += sizeof(T);
    return v;
  }
  std::string str() {
    std::int32_t n = val<std::int32_t>();
    if (n < 0) throw Error(1, ".osh: negative string length");
    need(size_t(n));
    std::string s(b_.data() + p_, size_t(n));
    p_ += size_t(n);
    return s;
  }
  // one array's bytes and item count: a view into the file buffer, or the
  // decompressed bytes (held in *owned)
  const char* array(int esize, bool compressed, LO* n_out, std::vector<char>* owned) {
    LO n = val<LO>();
    if (n < 0) throw Error(1, ".osh: negative array size");
    size_t nb = size_t(n) * size_t(esize);
    *n_out = n;
    if (!compressed) {
      need(nb);
      const char* p = b_.data() + p_;
      p_ += nb;
      return p;
    }
    std::int64_t cb = val<std::int64_t>();
    if (cb < 0) throw Error(1, ".osh: negative compressed size");
    need(size_t(cb));
    const Zlib& z = zlib();
    if (!z.ok()) throw Error(1, ".osh: compressed file and no zlib on this system");
    owned->resize(nb);
    unsigned long got = nb;
    int rc = z.uncompress(reinterpret_cast<unsigned char*>(owned->data()), &got,
                          reinterpret_cast<const unsigned char*>(b_.data() + p_), size_t(cb));
    if (rc != 0 || got != nb) throw Error(1, ".osh: zlib stream does not match its array");
    p_ += size_t(cb);
    return owned->data();
  }
  bool done() const { return p_ == b_.size(); }

 private:
  void need(size_t n) {
    if (p_ + n > b_.size()) throw Error(1, ".osh: file ends early");
  }
  std::vector<char> b_;
  size_t p_ = 0;
};

// one array from host bytes to the device, in one copy
template <class T>
Arr<T> upload(const char* bytes, LO n) {
  Arr<T> a(n);
  if (n)
    OHG_CUDA(cudaMemcpyAsync(a.data(), bytes, size_t(n) * sizeof(T), cudaMemcpyHostToDevice,
                             ctx().stream));
  return a;
}

void write_text(const std::string& path, int v) {
  std::ofstream f(path);
  if (!f) throw Error(1, "cannot write " + path);
  f << v << '\n';
}
int read_int_file(const std::string& path) {
  std::ifstream f(path);
  if (!f) return -1;
  int v = -1;
  f >> v;
  if (!f) throw Error(1, "cannot read an integer from " + path);
  return v;
}

// the tags of dimension d in the order the reference leaves them: a fresh
// box lists its coordinates first, a rebuilt mesh after the classification
// (transfer order); lengths and qualities come last, as they are added last
std::vector<std::string> canonical_order(const Mesh& m, int d) {
  std::vector<std::string> o;
  if (d == 0 && !m.rebuilt) o.push_back("coordinates");
  o.push_back("global");
  if (m.class_id[d].size() || m.nents[d] == 0) o.push_back("class_id");
  if (m.class_dim[d].size() || m.nents[d] == 0) o.push_back("class_dim");
  if (d == 0 && m.rebuilt) o.push_back("coordinates");
  if (d == 0 && m.metric.size()) o.push_back("metric");
  if (d == 1 && m.has_length) o.push_back("length");
  if (d == m.dim && m.has_quality) o.push_back("quality");
  return o;
}

bool is_iota(const std::vector<std::int64_t>& g) {
  for (size_t i = 0; i < g.size(); ++i)
    if (g[i] != std::int64_t(i)) return false;
  return true;
}

}  // namespace

bool zlib_available() { return zlib().ok(); }

// binary::write (src/Omega_h_file.cpp:355-396 and :488-505 for the directory)
void write_osh(Mesh& m, const std::string& dir, bool compress) {
  if (compress && !zlib().ok()) throw Error(1, ".osh: compression asked for and no zlib found");
  Out o(compress);
  o.bytes(kMagic, 2);
  o.val<I8>(I8(compress ? 1 : 0));
  o.val<I8>(0);  // simplex family
  o.val<I8>(I8(m.dim));
  o.val<std::int32_t>(1);  // one part
  o.val<std::int32_t>(0);
  o.val<I8>(I8(m.parting));
  o.val<std::int32_t>(m.parting ? 1 : 0);
  o.val<I8>(0);  // no inertial bisection hints
  o.val<LO>(m.nents[0]);
  for (int d = 1; d <= m.dim; ++d) {
    const Adj& a = m.adj.at({d, d - 1});
    o.device_array(a.ab2b);
    if (d > 1) o.device_array(a.codes);
  }
  for (int d = 0; d <= m.dim; ++d) {
    std::vector<std::string> order = m.tag_order[d].empty() ? canonical_order(m, d) : m.tag_order[d];
    if (!m.tag_order[d].empty()) {
      // tags added since the file was read go last
      for (const std::string& n : canonical_order(m, d))
        if (std::find(order.begin(), order.end(), n) == order.end()) order.push_back(n);
    }
    // known tags without data (lengths and qualities not measured, as in
    // a clone) are not written
    order.erase(std::remove_if(order.begin(), order.end(),
                               [&](const std::string& n) {
                                 for (const Mesh::Tag& t : m.extra_tags)
                                   if (t.dim == d && t.name == n) return false;
                                 return (n == "length" && !m.has_length) ||
                                        (n == "quality" && !m.has_quality) ||
                                        (n == "metric" && m.metric.size() == 0);
                               }),
                order.end());
    o.val<std::int32_t>(std::int32_t(order.size()));
    for (const std::string& name : order) {
      const Mesh::Tag* extra = nullptr;
      for (const Mesh::Tag& t : m.extra_tags)
        if (t.dim == d && t.name == name) extra = &t;
      o.str(name);
      if (extra) {
        o.val<I8>(I8(extra->ncomps));
        o.val<I8>(I8(extra->type));
        std::vector<I8> h = to_host(extra->bytes);
        o.array(h.data(), LO(h.size() / size_t(type_size(extra->type))), type_size(extra->type));
      } else if (name == "global") {
        o.val<I8>(1);
        o.val<I8>(T_I64);
        std::vector<std::int64_t> g(size_t(m.nents[d]));
        for (LO i = 0; i < m.nents[d]; ++i) g[size_t(i)] = i;
        o.array(g.data(), m.nents[d], 8);
      } else if (name == "coordinates") {
        o.val<I8>(I8(m.dim));
        o.val<I8>(T_F64);
        o.device_array(m.coords);
      } else if (name == "metric") {
        o.val<I8>(I8(m.mcomp()));
        o.val<I8>(T_F64);
        o.device_array(m.metric);
      } else if (name == "class_id") {
        o.val<I8>(1);
        o.val<I8>(T_I32);
        o.device_array(m.class_id[d]);
      } else if (name == "class_dim") {
        o.val<I8>(1);
        o.val<I8>(T_I8);
        o.device_array(m.class_dim[d]);
      } else if (name == "length") {
        o.val<I8>(1);
        o.val<I8>(T_F64);
        o.device_array(m.length);
      } else if (name == "quality") {
        o.val<I8>(1);
        o.val<I8>(T_F64);
        o.device_array(m.quality);
      } else {
        throw Error(1, ".osh: no data for tag " + name);
      }
    }
  }
  o.val<std::int32_t>(std::int32_t(m.class_sets.size()));
  for (const auto& kv : m.class_sets) {  // by name, as the reference's std::map
    o.str(kv.first);
    o.val<std::int32_t>(std::int32_t(kv.second.size()));
    for (const auto& p : kv.second) {
      o.val<std::int32_t>(p.first);
      o.val<std::int32_t>(p.second);
    }
  }
  o.val<I8>(0);  // no parents
  mkdir(dir.c_str(), 0755);
  struct stat st;
  if (stat(dir.c_str(), &st) != 0 || !S_ISDIR(st.st_mode))
    throw Error(1, "cannot create directory " + dir);
  std::ofstream f(dir + "/0.osh", std::ios::binary);
  if (!f) throw Error(1, "cannot write " + dir + "/0.osh");
  f.write(o.buf().data(), std::streamsize(o.buf().size()));
  if (!f) throw Error(1, "write failed: " + dir + "/0.osh");
  f.close();
  write_text(dir + "/nparts", 1);
  write_text(dir + "/version", kLatestVersion);
}

// binary::read (src/Omega_h_file.cpp:398-450, read_meta :226-272, read_tag
// :296-332, read_sets :348-356), one part
Mesh read_osh(const std::string& dir) {
  int nparts = read_int_file(dir + "/nparts");
  if (nparts != 1) throw Error(1, ".osh: " + dir + " has " + std::to_string(nparts) +
                                      " parts; one part is read");
  int version = read_int_file(dir + "/version");
  if (version < 1 || version > kLatestVersion)
    throw Error(1, ".osh: unsupported version " + std::to_string(version));
  std::ifstream f(dir + "/0.osh", std::ios::binary | std::ios::ate);
  if (!f) throw Error(1, "cannot read " + dir + "/0.osh");
  std::streamsize fsize = f.tellg();
  f.seekg(0);
  std::vector<char> b(static_cast<size_t>(fsize > 0 ? fsize : 0));
  if (fsize > 0 && !f.read(b.data(), fsize)) throw Error(1, "cannot read " + dir + "/0.osh");
  In in(std::move(b));
  unsigned char mg0 = (unsigned char)in.val<char>(), mg1 = (unsigned char)in.val<char>();
  if (mg0 != kMagic[0] || mg1 != kMagic[1]) throw Error(1, ".osh: bad magic number");
  bool comp = in.val<I8>() != 0;
  Mesh m;
  if (version >= 7 && in.val<I8>() != 0) throw Error(1, ".osh: only simplex meshes are read");
  m.dim = in.val<I8>();
  if (m.dim != 2 && m.dim != 3) throw Error(1, ".osh: dimension must be 2 or 3");
  std::int32_t csize = in.val<std::int32_t>(), crank = in.val<std::int32_t>();
  if (csize != 1 || crank != 0) throw Error(1, ".osh: written by more than one rank");
  m.parting = in.val<I8>() == 1 ? 1 : 0;
  if (version >= 3) in.val<std::int32_t>();
  if (in.val<I8>()) {
    std::int32_t naxes = in.val<std::int32_t>();
    for (std::int32_t i = 0; i < 3 * naxes; ++i) in.val<double>();
  }
  if (version < 6) in.val<I8>();
  m.nents[0] = in.val<LO>();
  for (int d = 1; d <= m.dim; ++d) {
    Adj a;
    LO n;
    std::vector<char> owned;
    const char* ab = in.array(4, comp, &n, &owned);
    a.ab2b = upload<LO>(ab, n);
    if (d > 1) {
      const char* cb = in.array(1, comp, &n, &owned);
      a.codes = upload<I8>(cb, n);
      a.has_codes = true;
    }
    m.set_ents(d, std::move(a));
  }
  for (int d = 0; d <= m.dim; ++d) {
    std::int32_t ntags = in.val<std::int32_t>();
    for (std::int32_t i = 0; i < ntags; ++i) {
      std::string name = in.str();
      int ncomps = in.val<I8>(), type = in.val<I8>();
      if (version < 5) {
        in.val<I8>();
        if (version >= 2) in.val<I8>();
      }
      LO n;
      std::vector<char> owned;
      const char* bytes = in.array(type_size(type), comp, &n, &owned);
      size_t nbytes = size_t(n) * size_t(type_size(type));
      if (n != LO(std::int64_t(m.nents[d]) * ncomps))
        throw Error(1, ".osh: tag " + name + " has the wrong size");
      m.tag_order[d].push_back(name);
      bool known = true;
      if (name == "coordinates" && d == 0 && type == T_F64 && ncomps == m.dim) {
        m.coords = upload<double>(bytes, n);
      } else if (name == "metric" && d == 0 && type == T_F64 &&
                 (ncomps == m.mcomp() || ncomps == 1)) {
        m.metric = upload<double>(bytes, n);
        m.metric_comps = ncomps == 1 ? 1 : 0;
      } else if (name == "class_id" && type == T_I32 && ncomps == 1) {
        m.class_id[d] = upload<LO>(bytes, n);
      } else if (name == "class_dim" && type == T_I8 && ncomps == 1) {
        m.class_dim[d] = upload<I8>(bytes, n);
      } else if (name == "length" && d == 1 && type == T_F64 && ncomps == 1) {
        m.length = upload<double>(bytes, n);
        m.has_length = true;
      } else if (name == "quality" && d == m.dim && type == T_F64 && ncomps == 1) {
        m.quality = upload<double>(bytes, n);
        m.has_quality = true;
      } else if (name == "global" && type == T_I64 && ncomps == 1) {
        std::vector<std::int64_t> g(static_cast<size_t>(n));
        if (n) std::memcpy(g.data(), bytes, nbytes);
        known = is_iota(g);  // one rank numbers 0..n-1; anything else is kept as is
      } else {
        known = false;
      }
      if (!known) {
        Mesh::Tag t{d, ncomps, type, name, upload<I8>(bytes, LO(nbytes))};
        m.extra_tags.push_back(std::move(t));
      }
    }
  }
  if (version >= 8) {
    std::int32_t nsets = in.val<std::int32_t>();
    for (std::int32_t i = 0; i < nsets; ++i) {
      std::string name = in.str();
      std::int32_t np = in.val<std::int32_t>();
      auto& v = m.class_sets[name];
      for (std::int32_t j = 0; j < np; ++j) {
        int cd = in.val<std::int32_t>();
        int id = in.val<std::int32_t>();
        v.push_back({cd, id});
      }
    }
  }
  if (version >= 9 && in.val<I8>()) throw Error(1, ".osh: meshes with parent links are not read");
  if (!in.done()) throw Error(1, ".osh: bytes after the mesh");
  // a file in the order a rebuild leaves the vertex tags is marked rebuilt,
  // so that tags added later follow that order's rules
  const auto& o0 = m.tag_order[0];
  auto pos = [&](const char* s) {
    return std::find(o0.begin(), o0.end(), std::string(s)) - o0.begin();
  };
  m.rebuilt = pos("coordinates") > pos("class_dim") && pos("class_dim") < LO(o0.size());
  return m;
}

}  // namespace ohg
