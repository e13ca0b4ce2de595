// The per-pass adapt operators on a device-resident mesh.
#pragma once
#include "ohg_mesh.cuh"

namespace ohg {

struct AdaptOpts {
  double min_length_desired, max_length_desired, max_length_allowed;
  double min_quality_allowed, min_quality_desired;
  int nsliver_layers = 4;
  explicit AdaptOpts(int dim);  // src/Omega_h_adapt.cpp:52-85
};

struct PassStats {
  int did_refine = 0, did_coarsen = 0, did_swap = 0;
  LO nelems_in = 0, nelems_out = 0;
  LO refine_keys = 0, coarsen_keys = 0, swap_keys = 0;
  int indset_rounds = 0;
  double min_quality = 0;
  float ms_refine = 0, ms_coarsen = 0, ms_swap = 0;
};

// independent set over a conflict graph (src/Omega_h_indset.cpp,
// src/Omega_h_indset_inline.hpp); quality ties broken by entity number,
// which is the global number on one device.  No host wait: the call's
// sweep count is added to the context's device counter d_indset_sweeps.
Arr<I8> find_indset(const Adj& graph, LO n, const Arr<double>& quality, const Arr<I8>& cands);
Arr<I8> find_indset(Mesh& m, int d, const Arr<double>& quality, const Arr<I8>& cands);

// stage kernels (each fills caller memory of the stated size)
void refine_qualities(Mesh& m, const LO* cands2edges, LO n, const double* midmetrics,
                      double* out);
void check_collapse_class(Mesh& m, const LO* c2e, LO n, const I8* codes_in, I8* codes_out);
void check_collapse_exposure(Mesh& m, const LO* c2e, LO n, const I8* codes_in, I8* codes_out);
void prevent_coarsen_overshoot(Mesh& m, double max_length, const LO* c2e, LO n,
                               const I8* codes_in, I8* codes_out);
void coarsen_qualities(Mesh& m, const LO* c2e, LO n, const I8* codes, double* out2);
// FP32 enclosures of the FP64 quality of arbitrary vertex 4-tuples and of
// the FP64 metric length of vertex pairs, with the FP64 values (3D)
void screen_tets(Mesh& m, const LO* tv2v, LO n, float* lo, float* hi, double* exact);
void screen_tets_face(Mesh& m, const LO* tv2v, LO n, int slot, bool cubed, float* lo, float* hi,
                      double* exact);
void screen_edges(Mesh& m, const LO* ev2v, LO n, float* lo, float* hi, double* exact);
void choose_rails(Mesh& m, const LO* c2e, LO n, const I8* codes, const double* quals2,
                  I8* vert_cands, double* vert_quals, GO* vert_rails);
Arr<I8> mark_sliver_layers(Mesh& m, double ceil, int nlayers);
// swap2d_qualities (src/Omega_h_swap2d_qualities.cpp:15-81)
void swap2d_qualities(Mesh& m, double max_length_allowed, const LO* c2e, LO n, double* quals);
// device bytes held by a mesh (each buffer once)
std::size_t mesh_device_bytes(const Mesh& m);
// swap3d::find_loop per edge: ring size (0 outside 3..7), the edge's two
// vertices, and up to 7 loop vertices per edge
void swap3d_find_loops(Mesh& m, const LO* edges, LO n, int* sizes, LO* eev2v, LO* loop_verts);
void swap3d_qualities(Mesh& m, double max_length_allowed, const LO* c2e, LO n, double* quals,
                      I8* configs);

bool refine_by_size(Mesh& m, const AdaptOpts& o, PassStats* st);
bool coarsen_by_size(Mesh& m, const AdaptOpts& o, PassStats* st);
bool coarsen_slivers(Mesh& m, const AdaptOpts& o, PassStats* st);

// outcome of a full adapt(): whether the mesh needed work, how many times
// each operator changed it, and whether the quality goal was reached
struct AdaptResult {
  bool did = false;
  bool quality_satisfied = false;
  int refines = 0, coarsens = 0, swaps = 0, sliver_coarsens = 0, length_rounds = 0;
};
AdaptResult adapt(Mesh& m, const AdaptOpts& o);
bool swap_edges(Mesh& m, const AdaptOpts& o, PassStats* st);
// refine -> coarsen -> swap when min quality < min_quality_desired
PassStats adapt_pass(Mesh& m, const AdaptOpts& o);

}  // namespace ohg
