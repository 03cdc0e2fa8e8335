// facade_main.cpp -- drives the C++ drop-in (robartsvtk_gb300/csrc/hmf_segmentation.hpp)
// the way a VTK-free caller would: build the filter, set the tree, the inputs
// and the parameters, Update(), read GetOutputDataObject(leaf).  Used by
// tests/test_cpp_facade.py.
//
// usage: facade_main <dir>   (reads <dir>/spec.txt, writes <dir>/out_<leaf>.raw
//                             and <dir>/status.txt)
// spec.txt:
//   vx vy vz
//   n parent_0 .. parent_{n-1}
//   iterations step cc semantics
//   n_alpha  (node alpha) x n_alpha
//   n_data   (node file)  x n_data
//   n_smooth (node file)  x n_smooth
//   [max_gpu_usage [k2]]  (optional: SetMaxGPUUsage, an out-of-core solve when
//                          >= 0; then ContinueUpdate with k2 iterations)
#include <cstdio>
#include <fstream>
#include <iostream>
#include <map>
#include <string>
#include <vector>

#include "hmf_segmentation.hpp"

static std::vector<float> read_raw(const std::string& path, size_t n) {
  std::vector<float> v(n);
  std::FILE* f = std::fopen(path.c_str(), "rb");
  if (!f || std::fread(v.data(), sizeof(float), n, f) != n) {
    std::cerr << "cannot read " << path << "\n";
    std::exit(2);
  }
  std::fclose(f);
  return v;
}

int main(int argc, char** argv) {
  if (argc != 2) {
    std::cerr << "usage: facade_main <dir>\n";
    return 2;
  }
  const std::string dir = argv[1];
  std::ifstream spec(dir + "/spec.txt");
  int dims[3];
  int n;
  spec >> dims[0] >> dims[1] >> dims[2] >> n;
  std::vector<int> parent(n);
  for (int& p : parent) spec >> p;
  int iterations, semantics;
  float step, cc;
  spec >> iterations >> step >> cc >> semantics;
  const size_t nvox = (size_t)dims[0] * dims[1] * dims[2];

  hmf::HierarchicalMaxFlowSegmentation filter;
  filter.SetHierarchy(parent);
  filter.SetNumberOfIterations(iterations);
  filter.SetStepSize(step);
  filter.SetCC(cc);
  filter.SetSemantics(semantics);
  int count;
  spec >> count;
  for (int k = 0; k < count; ++k) {
    int node;
    double alpha;
    spec >> node >> alpha;
    filter.AddSmoothnessScalar(node, alpha);
  }
  std::map<int, std::vector<float>> inputs;  // kept alive: the filter borrows them
  spec >> count;
  for (int k = 0; k < count; ++k) {
    int node;
    std::string file;
    spec >> node >> file;
    inputs[node] = read_raw(dir + "/" + file, nvox);
    filter.SetDataInputDataObject(node, inputs[node].data(), dims);
  }
  spec >> count;
  for (int k = 0; k < count; ++k) {
    int node;
    std::string file;
    spec >> node >> file;
    inputs[-1 - node] = read_raw(dir + "/" + file, nvox);
    filter.SetSmoothnessInputDataObject(node, inputs[-1 - node].data(), dims);
  }
  double usage;
  int k2 = -1;
  if (spec >> usage) {
    filter.SetMaxGPUUsage(usage);
    if (!(spec >> k2)) k2 = -1;
  }

  int rc = filter.Update();
  if (rc == 1 && k2 >= 0) {
    filter.SetNumberOfIterations(k2);
    rc = filter.ContinueUpdate();
  }
  std::ofstream status(dir + "/status.txt");
  status << rc << "\n" << filter.GetNumberOfOutputPorts() << "\n" << filter.GetLastError() << "\n";
  if (rc != 1) return 0;
  for (int leaf : filter.GetLeafOrder()) {
    const float* out = filter.GetOutputDataObject(leaf);
    std::FILE* f = std::fopen((dir + "/out_" + std::to_string(leaf) + ".raw").c_str(), "wb");
    std::fwrite(out, sizeof(float), nvox, f);
    std::fclose(f);
  }
  return 0;
}
