// Stand-in for the isosurface library's cube tables.  The boundary-site sweep
// never reads the cycle table, so the table is empty; coordmap lists the 8
// offsets of a unit cube's corners.  Test infrastructure only.
#pragma once

const int coordmap[8][3] = {{0, 0, 0}, {0, 0, 1}, {0, 1, 0}, {0, 1, 1},
                            {1, 0, 0}, {1, 0, 1}, {1, 1, 0}, {1, 1, 1}};

class Cycle {
public:
    int getLength() const { return 0; }
    int getEdge(int) const { return 0; }
};

class CycleList {
    Cycle c_;

public:
    int getLength() const { return 0; }
    Cycle* getFirst() { return &c_; }
    void rotateLeft() {}
};

class Cube {
    CycleList l_;

public:
    explicit Cube(const char*) {}
    CycleList* getCycle(int) { return &l_; }
};
