// Reads a .vtu or .vtt with include/pn_vtu.hpp and prints one line per array:
// "<section> <name> <count> <sum> <sum of squares>", then writes the grid
// back out (argv[2], .vtu) so the Python reader can check the writer.
#include <cstdio>
#include <string>

#include "pn_vtu.hpp"

static void dump(const char *sec, const pnvtu::DataArray &a) {
  double s = 0, q = 0;
  for (double v : a.values) {
    s += v;
    q += v * v;
  }
  std::printf("%s %s %zu %.17g %.17g\n", sec, a.name.c_str(), a.values.size(), s, q);
}

int main(int argc, char **argv) {
  if (argc < 2) return 2;
  const std::string path = argv[1];
  try {
    if (path.size() > 4 && path.substr(path.size() - 4) == ".vtt") {
      const pnvtu::Table t = pnvtu::read_vtt(path);
      for (auto &a : t.columns) dump("RowData", a);
      for (auto &a : t.field_data) dump("FieldData", a);
      return 0;
    }
    const pnvtu::Grid g = pnvtu::read_vtu(path);
    dump("Points", pnvtu::DataArray{"points", "Float64", 3, g.points});
    dump("Cells", pnvtu::DataArray{"connectivity", "Int64", 1, g.connectivity});
    dump("Cells", pnvtu::DataArray{"offsets", "Int64", 1, g.offsets});
    for (auto &a : g.point_data) dump("PointData", a);
    for (auto &a : g.cell_data) dump("CellData", a);
    for (auto &a : g.field_data) dump("FieldData", a);
    if (argc > 2) pnvtu::write_vtu(argv[2], g);
  } catch (const std::exception &e) {
    std::printf("error %s\n", e.what());
    return 1;
  }
  return 0;
}
