// Link stubs for the OctreeVolume members that surfacing.cpp references on its
// octree branch.  The oracle only ever passes dense volumes, so none of these
// run.  TEST INFRASTRUCTURE.
#include <voxelcore/octree.h>

OctreeVolume::OctreeVolume() : m_max_res(0), m_root(nullptr), m_data(nullptr) {}
OctreeVolume::~OctreeVolume() {}
double OctreeVolume::getDataAt(int, int, int) { return 0.0; }
double OctreeVolume::getDataAt(int, int, int) const { return 0.0; }
void OctreeVolume::getBoundaryVoxels(vector<ivec3>& _v) const { _v.clear(); }
void OctreeVolume::walkTree(Walker*) {}
void OctreeVolume::walkSubtree(Walker*, OctreeNode*, const ivec3&, int) {}
