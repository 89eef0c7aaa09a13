/* Stand-in for tetgen's I/O struct (not used by the compiled functions). */
#pragma once
struct tetgenio {
  double* pointlist = 0; int numberofpoints = 0; int* trifacelist = 0; int numberoffacets = 0;
  int* tetrahedronlist = 0; int numberoftetrahedra = 0; double* tetrahedronattributelist = 0;
  bool load_tetmesh(char*, bool) { return false; }
};
