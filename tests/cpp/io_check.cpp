// Writes the file formats of include/lc2_io.hpp for the CPU tests:
//   io_check <dir>  ->  <dir>/g.png (37 x 23 grey ramp), <dir>/v.nrrd
//   (4 x 3 x 2 volume, values 0..23, sheared directions), <dir>/m.mat.
#include <cstdint>
#include <string>
#include <vector>

#include "lc2_io.hpp"

int main(int argc, char** argv) {
  if (argc != 2) return 2;
  const std::string dir = argv[1];
  std::vector<uint8_t> px(37 * 23);
  for (int y = 0; y < 23; ++y)
    for (int x = 0; x < 37; ++x) px[y * 37 + x] = (uint8_t)((x * 7 + y * 11) & 0xff);
  lc2io::write_png_gray8(dir + "/g.png", 37, 23, px.data());
  std::vector<float> v(24);
  for (int i = 0; i < 24; ++i) v[i] = 0.5f * i;
  lc2io::NrrdHeader h{{4, 3, 2}, {{1.5f, 0.25f, 0.0f}, {0.0f, 2.0f, 0.0f}, {0.0f, 0.0f, 3.0f}},
                      {-10.0f, 20.5f, 3.25f}};
  lc2io::write_nrrd(dir + "/v.nrrd", h, v.data());
  const float m[16] = {1, 0, 0, 2.5f, 0, 0.5f, 0, -1, 0, 0, 2, 0.125f, 0, 0, 0, 1};
  lc2io::write_matrix(dir + "/m.mat", m, 4, 4);
  return 0;
}
