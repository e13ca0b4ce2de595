// A drop-in for the adapt pass of Omega_h on one GB300, for C++ callers that
// hold an Omega_h::Mesh.  It keeps the reference's Mesh and AdaptOpts types:
// the mesh's arrays go into the C ABI of include/ohg.h (device or host
// memory, whichever the reference's build keeps them in), the pass runs on
// the GPU, and the Mesh is rebuilt from the result with the reference's own
// Mesh API (copy_meta, set_verts, set_ents, add_tag), as its operators
// rebuild it (src/Omega_h_modify.cpp).
//
// Compile this file together with the reference's headers and link it with
// libohg.so; nothing here is compiled into libohg.so itself.
#ifndef OMEGA_H_ADAPT_GB300_HPP
#define OMEGA_H_ADAPT_GB300_HPP

#include <Omega_h_adapt.hpp>
#include <Omega_h_mesh.hpp>

#include "ohg.h"

namespace Omega_h {

// One adapt pass: refine_by_size, coarsen_by_size, and swap_edges when the
// worst quality is below opts.min_quality_desired, as adapt() runs them
// (src/Omega_h_adapt.cpp:185-199).  Replaces *mesh with the result and
// returns whether any operator changed it.
bool adapt_pass_gb300(ohg_context* ctx, Mesh* mesh, AdaptOpts const& opts);

// The whole adapt() loop (src/Omega_h_adapt.cpp:272-288) for meshes without
// conservation tags or geometry.  Replaces *mesh with the result and returns
// whether anything changed, as adapt() does.
bool adapt_gb300(ohg_context* ctx, Mesh* mesh, AdaptOpts const& opts);

// Both refuse (Omega_h_fail) a mesh they cannot carry through the pass
// without losing data: not a simplex mesh of dimension 2 or 3, more than one
// rank, or a tag other than coordinates, metric, class_dim, class_id,
// global, length and quality (the library transfers no user fields).

}  // namespace Omega_h

#endif
