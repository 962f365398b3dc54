// ncf_tfpws drop-in: S-transform time-frequency phase-weighted stack of
// every SourcePack group.
//
// Command line of the reference (native/tfpws/arguproc.c:4-177):
//   ncf_tfpws -I|--sourcepack-list <file> -O|--output-sourcepack <dir> [-G list]
//             [-S 001] [-M list] [-F lo/hi] [-T hz] [-B n] [--progress|--progress-file file]
// Output: tfpws.wNNN.{pack,tsv}, sourcepack_index.tsv, _SUCCESS; exit 0 / 1.
#include "stack_app.h"

static void usage() {
  fprintf(stderr,
          "\nUsage:\n"
          "  ncf_tfpws -I <sourcepack_inputs.txt> -O <output_dir> [options]\n\n"
          "  -I <file>   text file with one sourcepack_index.tsv path per line (--sourcepack-list)\n"
          "  -O <dir>    output directory for the TF-PWS SourcePack (--output-sourcepack)\n"
          "  -G <list>   comma-separated GPU worker IDs\n"
          "  -S <bin>    deprecated compatibility flag; TF-PWS bit must be 1 (e.g. 001)\n"
          "  -M <list>   optional comma-separated MiB caps, one per -G worker\n"
          "  -F <lo/hi>  only apply TF-PWS weighting inside this Hz band\n"
          "  -T <Hz>     raised-cosine taper width inside the -F band (default 5%% of the band)\n"
          "  -B <int>    pre-stack every <int> traces before TF-PWS (< 2: off)\n"
          "  --progress <file> write progress sidecar TSV\n");
}

int main(int argc, char** argv) {
  stackapp::Options o;
  o.tfpws = true;
  if (argc <= 1) {
    usage();
    return 1;
  }
  static struct option longopts[] = {{"progress", required_argument, 0, 1000},
                                     {"progress-file", required_argument, 0, 1000},
                                     {"sourcepack-list", required_argument, 0, 1003},
                                     {"output-sourcepack", required_argument, 0, 1004},
                                                                          {0, 0, 0, 0}};
  int c, idx = 0;
  while ((c = getopt_long(argc, argv, "I:O:G:S:B:M:F:T:", longopts, &idx)) != -1) {
    switch (c) {
      case 'I': o.list = optarg; break;
      case 'O': o.out = optarg; break;
      case 'G':
        o.gpus = optarg;
        if (o.gpus.empty()) {
          FXLOG_ERROR("invalid_gpu_list", "message=\"-G must not be empty\"");
          return 1;
        }
        break;
      case 'S':
        if (strlen(optarg) != 3 || strspn(optarg, "01") != 3) {
          FXLOG_ERROR("invalid_stack_selector", "value=\"%s\" expected=\"3-digit binary string, e.g. 001\"",
                      optarg);
          return 1;
        }
        if (optarg[2] != '1') {
          FXLOG_ERROR("invalid_stack_selector", "value=\"%s\" message=\"TF-PWS bit must be 1\"", optarg);
          return 1;
        }
        if (optarg[0] == '1' || optarg[1] == '1')
          FXLOG_WARN("ignored_stack_selector_bits",
                     "value=\"%s\" message=\"linear/PWS -S bits are ignored by TF-PWS\"", optarg);
        break;
      case 'M': o.mem_mib = optarg; break;
      case 'F':
        if (sscanf(optarg, "%lf/%lf", &o.fmin, &o.fmax) != 2 || o.fmin < 0.0 || o.fmax <= o.fmin) {
          FXLOG_ERROR("invalid_band_argument", "value=\"%s\" expected=\"fmin/fmax in Hz, e.g. 0.02/0.20\"",
                      optarg);
          return 1;
        }
        o.band_limited = 1;
        break;
      case 'T':
        o.taper_hz = atof(optarg);
        if (o.taper_hz < 0.0) {
          FXLOG_ERROR("invalid_band_taper", "value=\"%s\"", optarg);
          return 1;
        }
        break;
      case 'B':
        o.substack = atoi(optarg);
        if (o.substack < 2) o.substack = 1;
        break;
      case 1000: o.progress = optarg; break;
      case 1003: o.list = optarg; break;
      case 1004: o.out = optarg; break;
      default:
        FXLOG_ERROR("unknown_option", "option=-%c", optopt);
        usage();
        return 1;
    }
  }
  if (!o.list || !o.out) {
    FXLOG_ERROR("missing_sourcepack_io", "message=\"use -I/-O or --sourcepack-list/--output-sourcepack\"");
    usage();
    return 1;
  }
  return stackapp::run(o);
}
