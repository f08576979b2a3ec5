// stub_prelude.h — TEST INFRASTRUCTURE ONLY.  Empty stand-ins for the TBB and
// Boost headers that the reference's global headers include.  They let the
// reference's own arithmetic in base_cls_particle/particle.cpp compile for the
// checker without those libraries; nothing here is called by that code.
#pragma once
#include <cstddef>
#include <vector>
namespace tbb {}
namespace boost {
namespace serialization {
class access;
}
namespace mpi {}
struct listS {};
struct vecS {};
struct undirectedS {};
struct bidirectionalS {};
template <class... A>
struct adjacency_list {};
template <class G>
struct graph_traits {
  typedef int vertex_descriptor;
  typedef int edge_descriptor;
  typedef int vertex_iterator;
  typedef int edge_iterator;
  typedef int in_edge_iterator;
  typedef int out_edge_iterator;
  typedef int adjacency_iterator;
};
}  // namespace boost
