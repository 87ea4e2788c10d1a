// Drop-in `fringePreprocess` (src/fringePreprocess.cpp:287-365 of the reference):
//   fringePreprocess <motif_number>
//   fringePreprocess <n> <s0> <d0> <s1> <d1> ...
// Writes ./motif.mo (139 bytes) and ./motif.dot, printing the same progress
// and matching-order summary lines as the reference.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "fsgc.h"

static void print_order(const fsgc_matching_order& mo) {
  printf("starting from %c >= %d\n\n", 'A', mo.startdeg);
  for (int i = 0; i < mo.nodes - 1; i++) {
    printf("find %c >= %d\n", 'A' + i + 1, mo.destdeg[i]);
    printf(" connecting to");
    for (int j = 0; j <= i; j++)
      if (mo.list[i] & (1 << j)) printf(" %c", 'A' + j);
    if (mo.list[i] != ((2 << i) - 1)) {
      printf("\n skipping over");
      for (int j = 0; j <= i; j++)
        if (~mo.list[i] & (1 << j)) printf(" %c", 'A' + j);
    }
    printf("\n\n");
  }
  int anchors = 0;
  for (int i = 0; i < mo.anchorsets; i++) anchors |= mo.anch[i];
  printf("anchors:");
  for (int i = 0; i < mo.nodes; i++)
    if (anchors & (1 << i)) printf(" %c", 'A' + i);
  printf("\n\nanchor sets\n");
  for (int i = 0; i < mo.anchorsets; i++) {
    for (int j = 0; j < FSGC_MAX_CORE; j++)
      if (mo.anch[i] & (1 << j)) printf(" %c", 'A' + j);
    printf(": %d\n", mo.fcnt[i]);
  }
  printf("\n");
}

int main(int argc, char* argv[]) {
  printf("Fringe Preprocessor (fsgc, GB300-native)\n\n");
  if (argc < 2 || (argc % 2) != 0) {
    printf("USAGE: %s motif_number\n", argv[0]);
    printf("USAGE: %s number_of_nodes edge1_source edge1_destination ...\n\n", argv[0]);
    return -1;
  }
  int n = 0;
  std::vector<int> edges;
  if (argc == 2) {
    const int number = atoi(argv[1]);
    int ne = 0;
    if (fsgc_predefined_pattern(number, &n, nullptr, 0, &ne) != FSGC_OK) {
      printf("ERROR: unknown pattern\n\n");
      return -1;
    }
    edges.resize(2 * (size_t)ne);
    fsgc_predefined_pattern(number, &n, edges.data(), ne, &ne);
    printf("motif: %s\n", fsgc_predefined_name(number));
  } else {
    n = atoi(argv[1]);
    for (int p = 2; p + 1 < argc; p += 2) {
      edges.push_back(atoi(argv[p]));
      edges.push_back(atoi(argv[p + 1]));
    }
    printf("motif: user defined\n");
  }
  char err[256] = {0};
  fsgc_matching_order mo;
  const int st = fsgc_preprocess_log(n, edges.data(), (int)edges.size() / 2, &mo, err, sizeof(err), stdout);
  if (st != FSGC_OK) {
    fprintf(stderr, "ERROR: %s\n", err);
    return -1;
  }
  // motif.dot: the pattern with core vertices filled
  FILE* d = fopen("motif.dot", "w");
  if (d) {
    fprintf(d, "graph {\n");
    for (size_t e = 0; e + 1 < edges.size(); e += 2)
      fprintf(d, "  %d -- %d\n", edges[e] < edges[e + 1] ? edges[e] : edges[e + 1],
              edges[e] < edges[e + 1] ? edges[e + 1] : edges[e]);
    fprintf(d, "}\n");
    fclose(d);
  }
  print_order(mo);
  FILE* f = fopen("motif.mo", "wb");
  if (!f || fwrite(&mo, 1, sizeof(mo), f) != sizeof(mo)) {
    fprintf(stderr, "ERROR: could not write matching order to file\n");
    if (f) fclose(f);
    return -1;
  }
  fclose(f);
  printf("wrote matching order to file 'motif.mo'\n\n");
  return 0;
}
