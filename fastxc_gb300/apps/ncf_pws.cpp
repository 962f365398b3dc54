// ncf_pws drop-in: phase-weighted stack of every SourcePack group.
//
// Command line of the reference (native/pws/arguproc.c:5-129):
//   ncf_pws --index-list|--sourcepack-list <file> --output-dir|--output-sourcepack <dir>
//           [-G|--gpu-workers list] [-M|--gpu-memory-mib list] [-B|--substack-size n]
//           [-H|--staged-group-limit n] [--progress|--progress-file file]
// Output: pws.wNNN.{pack,tsv}, sourcepack_index.tsv, _SUCCESS; exit 0 / 1.
#include "stack_app.h"

static void usage() {
  fprintf(stderr,
          "\nUsage:\n"
          "  ncf_pws --index-list <file> --output-dir <dir> [options]\n\n"
          "  --index-list <file>            text file with one sourcepack_index.tsv path per line\n"
          "  --output-dir <dir>             output directory for pws pack shards and sourcepack_index.tsv\n"
          "  -G, --gpu-workers <list>       comma-separated GPU worker list (default: 0)\n"
          "  -M, --gpu-memory-mib <list>    comma-separated per-worker MiB caps; 0 means auto\n"
          "  -B, --substack-size <int>      average every <int> traces before PWS (< 2: off)\n"
          "  -H, --staged-group-limit <int> accepted for compatibility\n"
          "  --progress <file>              write progress sidecar TSV\n");
}

int main(int argc, char** argv) {
  stackapp::Options o;
  if (argc <= 1) {
    usage();
    return 1;
  }
  static struct option longopts[] = {
      {"progress", required_argument, 0, 1000},       {"progress-file", required_argument, 0, 1000},
      {"index-list", required_argument, 0, 1001},     {"sourcepack-list", required_argument, 0, 1001},
      {"output-dir", required_argument, 0, 1002},     {"output-sourcepack", required_argument, 0, 1002},
      {"gpu-workers", required_argument, 0, 'G'},     {"gpu-memory-mib", required_argument, 0, 'M'},
      {"substack-size", required_argument, 0, 'B'},   {"staged-group-limit", required_argument, 0, 'H'},
      {"host-group-limit", required_argument, 0, 'H'}, {0, 0, 0, 0}};
  int c, idx = 0;
  while ((c = getopt_long(argc, argv, "G:B:H:M:", longopts, &idx)) != -1) {
    switch (c) {
      case 'G':
        o.gpus = optarg;
        if (o.gpus.empty()) {
          FXLOG_ERROR("invalid_gpu_workers", "message=\"--gpu-workers/-G must not be empty\"");
          return 1;
        }
        break;
      case 'B':
        o.substack = atoi(optarg);
        if (o.substack < 2) o.substack = 1;
        break;
      case 'H':
        if (strtoull(optarg, nullptr, 10) < 1) {
          FXLOG_ERROR("invalid_staged_group_limit", "value=\"%s\"", optarg);
          return 1;
        }
        break;
      case 'M':
        o.mem_mib = optarg;
        if (o.mem_mib.empty()) {
          FXLOG_ERROR("invalid_gpu_memory_mib", "message=\"--gpu-memory-mib/-M must not be empty\"");
          return 1;
        }
        break;
      case 1000: o.progress = optarg; break;
      case 1001: o.list = optarg; break;
      case 1002: o.out = optarg; break;
      default:
        FXLOG_ERROR("unknown_option", "option=-%c", optopt);
        usage();
        return 1;
    }
  }
  if (!o.list || !o.out) {
    FXLOG_ERROR("missing_sourcepack_io", "index_list=\"%s\" output_dir=\"%s\"", o.list ? o.list : "",
                o.out ? o.out : "");
    usage();
    return 1;
  }
  return stackapp::run(o);
}
