// swift — command-line front end with the reference's flags and usage text
// (src/main.cu:42-431).  Single-end alignment runs the device pipeline:
// SSAHA seeding -> Smith-Waterman over 300-base windows -> best alignment per
// read -> default output records.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/swift_gb300.h"

static const char* usage_text() {
  return "\nUSAGE:\n"
         "   /path/to/swift -q <query fasta file> -r <reference fasta file> "
         "-o <output file> [optional parameters]\n\n"
         "DESCRIPTION:\n"
         "   Aligns multiple query sequences to multiple reference sequences "
         "using the Smith-Waterman algorithm.\n\n"
         "PARAMETERS:\n"
         "   -q     Query fasta file (required)\n"
         "   -q2    Paired query fasta file\n"
         "   -r     Reference fasta file (required)\n"
         "   -o     Output file (required)\n"
         "   -s     Query sequence size\n"
         "   -n     Number of queries\n"
         "   -l     Length of a seed (Default: 12)\n"
         "   -t     Threshold value used to ignore reference tuples\n"
         "   -m     Match score (Default: 2)\n"
         "   -M     Mismatch score (Default: -1)\n"
         "   -O     Gap open penalty (Default: -10)\n"
         "   -E     Gap extension penalty (Default: -1)\n"
         "   -cpu   Run program on CPU only\n"
         "   -f     Output format\n"
         "          0 - Default program output format. "
         "Output includes alignment, score, positions, and length.\n"
         "          1 - SAM format\n"
         "   -v     Print program version\n"
         "   -h     Print usage\n";
}

int main(int argc, char** argv) {
  const char *q = nullptr, *q2 = nullptr, *r = nullptr, *o = nullptr;
  swift_params p;
  swift_params_default(&p);
  // Phase 1 of the reference's GPU branch is search2Queries (lt13
  // seed-and-extend, src/main.cu:135-150); -seeder 0 selects the SSAHA
  // seeding of searchQueries3 instead (not a reference flag)
  p.seeder = 1;
  int cpu = 0;
  if (argc == 1) {
    printf("%s\n", usage_text());
    return 0;
  }
  for (int i = 1; i < argc; ++i) {
    const char* a = argv[i];
    const char* v = i + 1 < argc ? argv[i + 1] : nullptr;
    auto take = [&]() { ++i; return v ? v : ""; };
    if (!strcmp(a, "-q")) q = take();
    else if (!strcmp(a, "-q2")) q2 = take();
    else if (!strcmp(a, "-r")) r = take();
    else if (!strcmp(a, "-o")) o = take();
    else if (!strcmp(a, "-s")) p.qry_len = atoi(take());
    else if (!strcmp(a, "-n") || !strcmp(a, "-S") || !strcmp(a, "-N") || !strcmp(a, "-ms") ||
             !strcmp(a, "-MS")) take();
    else if (!strcmp(a, "-m")) p.match = atoi(take());
    else if (!strcmp(a, "-M")) p.mismatch = atoi(take());
    else if (!strcmp(a, "-O")) p.gap_open = atoi(take());
    else if (!strcmp(a, "-E")) p.gap_ext = atoi(take());
    else if (!strcmp(a, "-f")) p.out_format = atoi(take());
    else if (!strcmp(a, "-t")) p.ignore_thres = atoi(take());
    else if (!strcmp(a, "-l")) p.seed_len = atoi(take());
    else if (!strcmp(a, "-cpu")) cpu = 1;
    else if (!strcmp(a, "-seeder")) p.seeder = atoi(take());
    else if (!strcmp(a, "-v")) {
      printf("Version: %s\n", "0.11.2");
      return 0;
    } else {
      printf("%s\n", usage_text());
      return 0;
    }
  }
  if (!q || !r || !o) {
    printf("%s\n", usage_text());
    return 0;
  }
  if (q2 || cpu) {
    fprintf(stderr, "swift: %s is not supported by this build\n",
            q2 ? "paired-end alignment (-q2)" : "-cpu");
    return 2;
  }
  swift_ctx* ctx = nullptr;
  if (swift_ctx_create(0, nullptr, &ctx) != SWIFT_OK) {
    fprintf(stderr, "swift: no CUDA device\n");
    return 1;
  }
  int rc = swift_align_files(ctx, q, r, o, &p);
  if (rc != SWIFT_OK) fprintf(stderr, "swift: %s\n", swift_last_error(ctx));
  swift_ctx_destroy(ctx);
  return rc == SWIFT_OK ? 0 : 1;
}
