// Device-resident simplex mesh: the stored downward adjacencies, vertex
// fields, classification and the lazily derived adjacency cache
// (the roles of Omega_h::Mesh, src/Omega_h_mesh.hpp:36-177, and
// src/Omega_h_mesh.cpp:307-357).
#pragma once
#include "ohg_prims.cuh"

namespace ohg {

struct Adj {
  Arr<LO> a2ab, ab2b;
  Arr<I8> codes;
  bool has_a2ab = false, has_codes = false;
};

inline int simplex_degree(int from, int to) {
  static const int t[4][4] = {{1, -1, -1, -1}, {2, 1, -1, -1}, {3, 3, 1, -1}, {4, 6, 4, 1}};
  return t[from][to];
}

struct VertScreen;

struct Mesh {
  int dim = 3;
  LO nents[4] = {0, 0, 0, 0};
  Arr<double> coords;  // dim per vertex
  Arr<double> metric;  // 6 (3D) or 3 (2D) per vertex, packed symmetric
  Arr<I8> class_dim[4];
  Arr<LO> class_id[4];
  bool has_length = false, has_quality = false;
  Arr<double> length, quality;
  std::map<std::pair<int, int>, Adj> adj;
  // upward adjacencies whose rows are in no particular order, for the
  // consumers that do not depend on it (never returned by ask_adj)
  std::map<std::pair<int, int>, Adj> adj_any_order;
  // state the reference writes to .osh files: its partitioning mode (0
  // element-based, 1 ghosted: set by the operators as the reference's are),
  // whether the tags are in the order a rebuild leaves them, the named sets
  // of geometric model entities, tags this library does not model (kept
  // until the next rebuild), and the tag order of a file that was read
  int parting = 0;
  bool rebuilt = false;
  std::map<std::string, std::vector<std::pair<int, int>>> class_sets;
  struct Tag {
    int dim, ncomps, type;
    std::string name;
    Arr<I8> bytes;
  };
  std::vector<Tag> extra_tags;
  std::vector<std::string> tag_order[4];
  // the precision mode's per-vertex screening data, built on first use from
  // coords and metric; reset wherever those arrays are replaced
  std::shared_ptr<VertScreen> screen;

  // components of the vertex metric: the packed tensor (6 in 3D, 3 in 2D),
  // or 1 for an isotropic metric (metric_comps = 1)
  int metric_comps = 0;
  int mcomp() const { return metric_comps ? metric_comps : (dim == 3 ? 6 : 3); }
  LO nverts() const { return nents[0]; }
  LO nedges() const { return nents[1]; }
  LO nelems() const { return nents[dim]; }
  void set_ents(int d, Adj down);
  const Adj& ask_adj(int from, int to);
  const Adj& ask_down(int from, int to) { return ask_adj(from, to); }
  const Adj& ask_up(int from, int to) { return ask_adj(from, to); }
  const Arr<LO>& ask_verts_of(int d) { return ask_adj(d, 0).ab2b; }
  // the sorted upward adjacency if it is at hand, else one with its rows in
  // atomic order (no row sort)
  const Adj& ask_up_any_order(int from, int to);
  const Arr<double>& ask_lengths();
  const Arr<double>& ask_qualities();
  void drop_cache();  // forget derived adjacencies (keeps stored down ones)
};

// adjacency derivation (src/Omega_h_adj.cpp)
// sorted = false leaves each row in the order its atomics gave it
Adj invert_adj(const Adj& down, int nlows_per_high, LO nlows, bool sorted = true);
// reflect_down by a hash table of the low entities' vertex tuples (entities
// this library built: unique by construction); needs no upward adjacency
Adj reflect_down_hashed(const Arr<LO>& hv2v, LO nh, const Arr<LO>& lv2v, LO nl, int hd, int ld);
// check_unique: scan every candidate and report a second match (arrays from
// a caller); otherwise stop at the first
Adj reflect_down(const Arr<LO>& hv2v, LO nh, const Arr<LO>& lv2v, const Adj& v2l, int hd, int ld,
                 bool check_unique = false);
Adj transit(const Adj& h2m, const Adj& m2l, int hd, int ld, LO nh);
Arr<LO> form_uses(const Arr<LO>& hv2v, LO nh, int hd, int ld);
Arr<LO> find_unique(const Arr<LO>& hv2v, LO nh, int hd, int ld);

// construction: box mesh, Hilbert renumbering, box classification
Mesh build_box(int dim, int n);
Arr<GO> hilbert_keys(const Arr<double>& coords, LO n, int dim);
void hilbert_transpose_keys(const std::uint64_t* axes, LO n, int dim, int bits,
                            std::uint64_t* keys);
Arr<LO> hilbert_sort(const Arr<double>& coords, LO n, int dim);
void reorder_by_hilbert(Mesh& m);
void classify_box(Mesh& m, int n);
void apply_workload(Mesh& m, int n, std::uint64_t seed, int metric_kind);

// .osh files (src/Omega_h_file.cpp): the mesh to/from one part of the
// reference's binary format
void write_osh(Mesh& m, const std::string& dir, bool compress);
Mesh read_osh(const std::string& dir);
bool zlib_available();

// measurement kernels
void measure_edges_metric(Mesh& m, const LO* a2e, LO na, double* out);
void measure_qualities(Mesh& m, const LO* a2e, LO na, double* out);
// the same for elements given by vertex tuples (dim + 1 each)
void measure_qualities_tuples(Mesh& m, const LO* tuples, LO na, double* out);
void mident_metrics(Mesh& m, const LO* edges, LO n, double* out);

}  // namespace ohg
