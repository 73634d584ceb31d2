// Umbrella header standing in for trimesh2's TriMesh.h: the reference sources
// compiled for the oracle only need the vector, box and transform subset.
#pragma once
#include "Box.h"
#include "Vec.h"
#include "XForm.h"
