// swift — command-line front end with the reference's flags and usage text
// (src/main.cu:42-431).  Single-end alignment runs the device pipeline:
// seeding (lt13 seed-and-extend, as the reference's GPU branch, or SSAHA) ->
// Smith-Waterman over 300-base windows -> best alignment per read -> output
// records.  With -q2, the paired-end pipeline (src/main.cu:172-212).
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "../../include/swift_gb300.h"

static bool slurp(const char* path, std::vector<char>* out) {
  FILE* f = fopen(path, "rb");
  if (!f) return false;
  fseek(f, 0, SEEK_END);
  const long n = ftell(f);
  fseek(f, 0, SEEK_SET);
  out->resize(n > 0 ? (size_t)n : 0);
  const bool ok = n <= 0 || fread(out->data(), 1, (size_t)n, f) == (size_t)n;
  fclose(f);
  return ok;
}

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
  unsigned min_frag = 99, max_frag = 600;  // MIN/MAX_FRAG_SIZE (src/common.h:66-68)
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
    else if (!strcmp(a, "-n") || !strcmp(a, "-S") || !strcmp(a, "-N")) take();
    else if (!strcmp(a, "-ms")) min_frag = (unsigned)atoi(take());
    else if (!strcmp(a, "-MS")) max_frag = (unsigned)atoi(take());
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
  if (cpu) {
    fprintf(stderr, "swift: -cpu is not supported by this build\n");
    return 2;
  }
  swift_ctx* ctx = nullptr;
  if (swift_ctx_create(0, nullptr, &ctx) != SWIFT_OK) {
    fprintf(stderr, "swift: no CUDA device\n");
    return 1;
  }
  if (q2) {
    std::vector<char> ref, r1, r2;
    if (!slurp(r, &ref) || !slurp(q, &r1) || !slurp(q2, &r2)) {
      fprintf(stderr, "swift: cannot read an input file\n");
      swift_ctx_destroy(ctx);
      return 1;
    }
    swift_index* idx = nullptr;
    char* text = nullptr;
    size_t n = 0;
    int rc = swift_index_build(ctx, ref.data(), ref.size(), p.seed_len, p.ignore_thres, &idx);
    if (rc == SWIFT_OK)
      rc = swift_align_paired(ctx, idx, r1.data(), r1.size(), r2.data(), r2.size(), &p, min_frag,
                              max_frag, &text, &n, nullptr);
    if (rc == SWIFT_OK) {
      FILE* f = fopen(o, "wb");
      if (!f || (n && fwrite(text, 1, n, f) != n)) rc = SWIFT_E_ARG;
      if (f) fclose(f);
    }
    if (rc != SWIFT_OK) fprintf(stderr, "swift: %s\n", swift_last_error(ctx));
    swift_free(text);
    swift_index_destroy(idx);
    swift_ctx_destroy(ctx);
    return rc == SWIFT_OK ? 0 : 1;
  }
  int rc = swift_align_files(ctx, q, r, o, &p);
  if (rc != SWIFT_OK) fprintf(stderr, "swift: %s\n", swift_last_error(ctx));
  swift_ctx_destroy(ctx);
  return rc == SWIFT_OK ? 0 : 1;
}
