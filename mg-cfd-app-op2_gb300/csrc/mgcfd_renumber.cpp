// mgcfd_renumber: renumber a multigrid mesh once and write it back in the
// reference's input layout (input.dat + one HDF5 file per level,
// euler3d.cpp:243-312), so that the reordered mesh can be used by any
// consumer, the reference's own euler3d included.  This is the standalone
// form of the reference's -n option (op_renumber at euler3d.cpp:377).
//
//   mgcfd_renumber -i input.dat [-d dir] -o outdir [-p prefix]
//                  [-m spatial|rcm|none] [-l] [--legacy-datasets]
//
//   -i/-d   input deck and its directory (as euler3d -i/-d)
//   -l      read the legacy-mode datasets (as euler3d -l)
//   -o      output directory (must exist); writes <outdir>/input.dat and
//           <outdir>/<prefix>L<l>.h5
//   -m      node order (default spatial = Morton curve)
//   --legacy-datasets  also write the ".renumbered", "areas" and
//           "edge_weights.recalculated" datasets that euler3d -l reads
#include <getopt.h>

#include <cstdio>
#include <cstring>
#include <string>

#include "mgcfd_gb300.h"

namespace {

void usage() {
  std::fprintf(stderr,
               "Usage: mgcfd_renumber -i input.dat [-d dir] -o outdir [-p prefix] [-m spatial|rcm|none] [-l]\n"
               "                      [--legacy-datasets]\n");
}

int fail(const char* what) {
  std::fprintf(stderr, "mgcfd_renumber: %s: %s\n", what, mgcfd_last_error());
  return 1;
}

}  // namespace

int main(int argc, char** argv) {
  std::string input, dir, outdir, prefix = "renumbered_";
  int method = MGCFD_RENUMBER_SPATIAL, legacy_in = 0, legacy_out = 0;
  static option longopts[] = {{"input-file", required_argument, nullptr, 'i'},
                              {"input-directory", required_argument, nullptr, 'd'},
                              {"output-directory", required_argument, nullptr, 'o'},
                              {"prefix", required_argument, nullptr, 'p'},
                              {"method", required_argument, nullptr, 'm'},
                              {"legacy", no_argument, nullptr, 'l'},
                              {"legacy-datasets", no_argument, nullptr, 'L'},
                              {"help", no_argument, nullptr, 'h'},
                              {nullptr, 0, nullptr, 0}};
  int c;
  while ((c = getopt_long(argc, argv, "i:d:o:p:m:lh", longopts, nullptr)) != -1) {
    switch (c) {
      case 'i': input = optarg; break;
      case 'd': dir = optarg; break;
      case 'o': outdir = optarg; break;
      case 'p': prefix = optarg; break;
      case 'l': legacy_in = 1; break;
      case 'L': legacy_out = 1; break;
      case 'm':
        if (!std::strcmp(optarg, "spatial")) method = MGCFD_RENUMBER_SPATIAL;
        else if (!std::strcmp(optarg, "rcm")) method = MGCFD_RENUMBER_RCM;
        else if (!std::strcmp(optarg, "none")) method = MGCFD_RENUMBER_NONE;
        else { usage(); return 1; }
        break;
      default: usage(); return 1;
    }
  }
  if (input.empty() || outdir.empty()) { usage(); return 1; }
  mgcfd_host_mesh* mesh = nullptr;
  if (mgcfd_host_mesh_load(input.c_str(), dir.c_str(), legacy_in, &mesh) != MGCFD_OK) return fail("load");
  mgcfd_host_mesh* out = nullptr;
  int st = mgcfd_host_mesh_renumber(mesh, method, &out);
  mgcfd_host_mesh_destroy(mesh);
  if (st != MGCFD_OK) return fail("renumber");
  st = mgcfd_host_mesh_write(out, outdir.c_str(), prefix.c_str(), legacy_out);
  int nl = mgcfd_host_mesh_num_levels(out);
  mgcfd_host_mesh_destroy(out);
  if (st != MGCFD_OK) return fail("write");
  std::printf("Renumbered %d level(s) into %s/input.dat\n", nl, outdir.c_str());
  return 0;
}
