// TEST INFRASTRUCTURE: known-answer tool built from the reference's own
// SeparatorTree (src/rschol/datastructure/SeparatorTree.h/.cpp), compiled
// where the reference sources lie into oracle/_ref/ (see
// rank_structured_cholesky_gb300/_build.py, build_reference_tools).
//
// Builds the separator tree exactly as NestedDissection::
// ReorderNestedSeparators does (src/rschol/ordering/NestedDissection.cpp:
// 811-817: LONGEST_AXIS, the block size as the leaf size, FIXED separators
// of thickness 0, build(points, false, true), then orderNodes and
// leafRanges) and prints the point order and the leaf ranges.
//
//   stdin:  npts maxLeaf, then npts lines "x y z"
//   stdout: npts point indices in tree order, then nLeaves, then nLeaves
//           "first last" pairs
#include <cstdio>
#include <vector>

#include <rschol/datastructure/SeparatorTree.h>

// The point type the reference instantiates the tree with (Mesh::MeshPoint,
// src/rschol/mesh/Mesh.h:64-83): an index and a degenerate bounding box.
class KatPoint {
 public:
  KatPoint(int index, const VEC3F &x) : _index(index) {
    _bbox.setMinBound(x);
    _bbox.setMaxBound(x);
  }
  int index() const { return _index; }
  const BoundingBox &bbox() const { return _bbox; }

 private:
  int _index;
  BoundingBox _bbox;
};

int main() {
  int npts = 0, maxLeaf = 0;
  if (std::scanf("%d %d", &npts, &maxLeaf) != 2) return 2;
  std::vector<KatPoint *> pts;
  for (int i = 0; i < npts; ++i) {
    double x, y, z;
    if (std::scanf("%lf %lf %lf", &x, &y, &z) != 3) return 2;
    pts.push_back(new KatPoint(i, VEC3F(x, y, z)));
  }
  typedef SeparatorTree<KatPoint> PointTree;
  std::vector<KatPoint *> work(pts);
  PointTree tree(PointTree::LONGEST_AXIS, maxLeaf, PointTree::FIXED, 0.0);
  tree.build(work, false, true);
  work.clear();
  tree.orderNodes(work);
  for (size_t i = 0; i < work.size(); ++i) std::printf("%d\n", work[i]->index());
  std::vector<IndexRange> ranges;
  tree.leafRanges(ranges);
  std::printf("%d\n", (int)ranges.size());
  for (size_t i = 0; i < ranges.size(); ++i) std::printf("%d %d\n", ranges[i].first, ranges[i].second);
  for (size_t i = 0; i < pts.size(); ++i) delete pts[i];
  return 0;
}
