/*
 * tap_main_gpu.c - tap_frankwolfe_gpu: the reference's pthread CLI
 * (tap/tap_main.c:89-276) on the GPU library.  Same flags, same output:
 *
 *   tap_frankwolfe_gpu [-n threads] [-w flows] [-i iter] [-r relgap]
 *                      [-t tripmods] [-v] netfile tripsfile  > flows
 *
 * -n is accepted for compatibility (the solver runs on one GPU).  Set
 * TAPGPU_PRECISION=fp32 to run the shortest paths with FP32 costs.
 */
#include <errno.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include "tap_gpu.h"

static const int DEFAULT_ITERATION_LIMIT = 10000; /* tap/tap_main.c:80 */

static void usage(const char *progname)
{
  fprintf(stderr,
          "Usage: %s  [-n numthreads] [-w warmstart_flows_filename] [-t tripmods_filename] "
          "netfilename demandfilename\n"
          "  -n numthreads : number of threads to use (default %d)\n"
          "  -w warmsetart_flows_filename : warmstart from previous solution\n"
          "  -i iterations : terminate after this many iterations (default %d)\n"
          "  -r relgap     : terminate when relative gap <= relgap\n"
          "  -t tripmodsfilename : modifiy O-D demand data\n"
          "  -v : verbose - write status each iteration to stderr\n",
          progname, num_cores, DEFAULT_ITERATION_LIMIT);
  exit(1);
}

static int link_cmp(const void *a, const void *b) { return link_data_compar(a, b); }

int main(int argc, char *argv[])
{
  int c, target_iterations = 0, warm_start_mode = 0, verbose = 0, trip_mods_mode = 0;
  int num_trip_mods = 0, iterations = 0;
  double target_relgap = 0, total_cost = 0, relgap = 0, objvalue = 0;
  char *flows_input_filename = NULL, *trip_mods_filename = NULL;
  FILE *flows_input_fp = NULL, *net_fp, *demand_fp;
  trip_mod_t *trip_mods = NULL;
  demand_data_t **demands = NULL;
  long num_zones = 0;
  net_data_t net;

  num_cores = (unsigned)sysconf(_SC_NPROCESSORS_ONLN);
  num_threads = num_cores;
  while ((c = getopt(argc, argv, "n:w:i:r:t:v")) != -1) {
    switch (c) {
      case 'n':
        if (atoi(optarg) < 1) {
          fprintf(stderr, "number of threads must be >= 1\n");
          usage(argv[0]);
        }
        num_threads = (unsigned)atoi(optarg);
        break;
      case 'w':
        flows_input_filename = optarg;
        warm_start_mode = 1;
        break;
      case 'i':
        if (atoi(optarg) < 1) {
          fprintf(stderr, "iteration target must be >= 1\n");
          usage(argv[0]);
        }
        target_iterations = atoi(optarg);
        break;
      case 'r':
        if (atof(optarg) <= 0) {
          fprintf(stderr, "relative gap must be positive\n");
          usage(argv[0]);
        }
        target_relgap = atof(optarg);
        break;
      case 't':
        trip_mods_filename = optarg;
        trip_mods_mode = 1;
        break;
      case 'v': verbose = 1; break;
      default: usage(argv[0]); break;
    }
  }
  if (argc - optind != 2) usage(argv[0]);
  if (target_relgap <= 0 && target_iterations <= 0) target_iterations = DEFAULT_ITERATION_LIMIT;

  if (trip_mods_mode) {
    FILE *fp = fopen(trip_mods_filename, "r");
    if (!fp) {
      fprintf(stderr, "error opening trips modifications file %s: %s\n", trip_mods_filename,
              strerror(errno));
      exit(1);
    }
    if (parse_trip_mod_file(fp, &trip_mods, &num_trip_mods) != 0) {
      fprintf(stderr, "parse trip mods file %s failed\n", trip_mods_filename);
      exit(1);
    }
    fclose(fp);
  }
  if (!(net_fp = fopen(argv[optind], "r"))) {
    fprintf(stderr, "error opening net file %s: %s\n", argv[optind], strerror(errno));
    exit(1);
  }
  if (!(demand_fp = fopen(argv[optind + 1], "r"))) {
    fprintf(stderr, "error opening trips file %s: %s\n", argv[optind + 1], strerror(errno));
    exit(1);
  }
  if (warm_start_mode && !(flows_input_fp = fopen(flows_input_filename, "r"))) {
    fprintf(stderr, "error opening flows input file %s: %s\n", flows_input_filename,
            strerror(errno));
    exit(1);
  }
  if (parse_net_file(net_fp, &net) != 0) {
    fprintf(stderr, "error parsing net file\n");
    exit(1);
  }
  fclose(net_fp);
  qsort(net.links, (size_t)net.num_links, sizeof(link_data_t), link_cmp);
  if (parse_trips_file(demand_fp, &demands, &num_zones) != 0) {
    fprintf(stderr, "error parsing trips file\n");
    return 1;
  }
  fclose(demand_fp);
  if (num_zones != net.num_zones)
    fprintf(stderr, "warning: %ld zones in net data but %ld in trips file\n", net.num_zones,
            num_zones);
  if (trip_mods_mode)
    for (int k = 0; k < num_trip_mods; k++)
      apply_trip_modification(demands, &trip_mods[k], num_zones);

  if (tap_frankwolfe(&net, demands, warm_start_mode, flows_input_fp, target_iterations,
                     target_relgap, stdout, &total_cost, &objvalue, &iterations, &relgap,
                     verbose) != 0) {
    fprintf(stderr, "failed\n");
    exit(1);
  }
  fprintf(stderr,
          "iterations = %d objective value = %.15f relative gap = %.15f total cost = %.15f\n",
          iterations, objvalue, relgap, total_cost);
  free(net.links);
  free(trip_mods);
  return 0;
}
