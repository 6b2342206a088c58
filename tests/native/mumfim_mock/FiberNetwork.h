// Stand-ins for the parts of mumfim's fiber network, its reactions and the
// APF mesh interface that the integration shim touches: a network is a list
// of vertices (points) and edges (vertex pairs) behind the apf::Mesh calls
// the shim makes, plus its reactions and scale factor. Test infrastructure
// only.
#ifndef MFG_TEST_FIBER_NETWORK_H
#define MFG_TEST_FIBER_NETWORK_H
#include <array>
#include <memory>
#include <vector>

namespace apf {
struct MeshEntity {
  int dim;
  int index;
};
struct MeshIterator {
  int dim;
  int next;
};
struct Vector3 {
  double v[3];
  double operator[](int k) const { return v[k]; }
  double& operator[](int k) { return v[k]; }
};
typedef MeshEntity* Downward[12];
struct Numbering {};

class Mesh {
 public:
  std::vector<std::array<double, 3>> points;
  std::vector<std::array<int, 2>> edges;
  std::vector<MeshEntity> verts, elems;
  void finalize() {
    verts.clear();
    elems.clear();
    for (int i = 0; i < static_cast<int>(points.size()); ++i) verts.push_back({0, i});
    for (int i = 0; i < static_cast<int>(edges.size()); ++i) elems.push_back({1, i});
  }
  MeshIterator* begin(int dim) { return new MeshIterator{dim, 0}; }
  MeshEntity* iterate(MeshIterator* it) {
    std::vector<MeshEntity>& v = it->dim == 0 ? verts : elems;
    return it->next < static_cast<int>(v.size()) ? &v[it->next++] : nullptr;
  }
  void end(MeshIterator* it) { delete it; }
  void getPoint(MeshEntity* e, int, Vector3& p) {
    for (int k = 0; k < 3; ++k) p[k] = points[e->index][k];
  }
  int getDownward(MeshEntity* e, int, Downward d) {
    d[0] = &verts[edges[e->index][0]];
    d[1] = &verts[edges[e->index][1]];
    return 2;
  }
};
inline Numbering* numberOwnedNodes(Mesh*, const char*) { return new Numbering(); }
inline int getNumber(Numbering*, MeshEntity* e, int, int) { return e->index; }
inline void destroyNumbering(Numbering* n) { delete n; }
}  // namespace apf

namespace mumfim {
struct FiberReaction {
  virtual ~FiberReaction() = default;
  double getYoungModulus() const noexcept { return E; }
  double getFiberArea() const noexcept { return fiber_area; }
  double getFiberDensity() const noexcept { return fiber_density; }
  double fiber_area = 0;
  double fiber_density = 0;
  double E = 0;
};
struct LinearReaction : FiberReaction {};
struct NonlinearReaction : FiberReaction {
  double B = 0;
  double length_ratio_trns = 0;
  double cmp_ratio_trns = 1.0;
};

class FiberNetwork {
 public:
  FiberNetwork(std::shared_ptr<apf::Mesh> mesh, std::vector<std::shared_ptr<FiberReaction>> r,
               double scale = 1.0)
      : mesh_(std::move(mesh)), reactions_(std::move(r)), scale_(scale) {}
  apf::Mesh* getNetworkMesh() const { return mesh_.get(); }
  const FiberReaction& getFiberReaction(size_t idx) const { return *reactions_[idx]; }
  double getScaleConversion() const noexcept { return scale_; }

 private:
  std::shared_ptr<apf::Mesh> mesh_;
  std::vector<std::shared_ptr<FiberReaction>> reactions_;
  double scale_;
};
}  // namespace mumfim
#endif
