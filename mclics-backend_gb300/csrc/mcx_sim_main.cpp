// mc_sim_gb300 <paramfile> -- command-line drop-in for the reference's
// ./mc_sim (src/main.cpp:63-83): removes the previous run's outputs from the
// working directory (src/main.cpp:43-61), then runs the parameter file's mode
// on the GPU through mcx_run_file.
#include <dirent.h>
#include <stdio.h>
#include <string.h>

#include "../../include/mcx.h"

static bool has_prefix(const char *s, const char *p) { return strncmp(s, p, strlen(p)) == 0; }
static bool has_suffix(const char *s, const char *x) {
  size_t a = strlen(s), b = strlen(x);
  return a >= b && strcmp(s + a - b, x) == 0;
}

int main(int argc, char **argv) {
  if (argc < 2) {
    fprintf(stderr, "usage: %s <paramfile>\n", argv[0]);
    return 5;
  }
  int removed = 0;
  if (DIR *d = opendir(".")) {
    while (struct dirent *e = readdir(d)) {
      const char *n = e->d_name;
      if (!strcmp(n, "ic.csv") || !strcmp(n, "po.dat") || (has_prefix(n, "po_r") && has_suffix(n, ".dat")) ||
          (has_prefix(n, "director_field_") && has_suffix(n, ".csv"))) {
        remove(n);
        removed++;
      }
    }
    closedir(d);
  }
  printf("  Removed %d output file(s) from a previous run.\n", removed);
  mcx_status st = mcx_run_file(argv[1], nullptr);
  if (st != MCX_OK) {
    fprintf(stderr, "  [ERROR] %s\n", mcx_last_error(nullptr));
    return (int)st + 10;
  }
  printf("  Simulation complete.\n");
  return 0;
}
