/*
 * Test infrastructure only: an option-string scanner for building the
 * reference SFF library (dacase/nabc src/sff) without flex.
 *
 * The reference generates lex.mmo.c from src/sff/mm_options.l with flex and
 * #includes it at the end of src/sff/sff.c (sff.c:2370), so this file is
 * compiled inside sff.c's translation unit and assigns sff.c's static option
 * variables (sff.c:68-199) directly.  It accepts the grammar of
 * mm_options.l:18-97 -- "key=value" or "key value" items separated by
 * commas, blanks, tabs or newlines -- echoes every accepted item as
 * "\tmm_options:  <item>" (mm_options.l:8) and exits(1) on an unknown key
 * (mm_options.l:99-111).
 *
 * Nothing in the product links this file; it only feeds oracle/_ref.
 */
#include <ctype.h>

#define MMO_DBL 0
#define MMO_INT 1
#define MMO_DIEL 2

typedef struct {
  const char *key;
  int kind;
  void *addr;
} mmo_entry_t;

static int mmo_lookup(const char *key, int *kind, void **addr)
{
  mmo_entry_t table[] = {
    {"cut", MMO_DBL, &cut}, {"cutnp", MMO_DBL, &cutnp},
    {"scnb", MMO_DBL, &scnb}, {"scee", MMO_DBL, &scee},
    {"ntpr", MMO_INT, &ntpr}, {"hcp", MMO_INT, &hcp},
    {"hcp_h1", MMO_DBL, &hcp_h1}, {"hcp_h2", MMO_DBL, &hcp_h2},
    {"hcp_h3", MMO_DBL, &hcp_h3}, {"dhcp", MMO_DBL, &dhcp},
    {"nscm", MMO_INT, &nscm}, {"nsnb", MMO_INT, &nsnb},
    {"nsnp", MMO_INT, &nsnp}, {"ntwx", MMO_INT, &ntwx},
    {"nchk", MMO_INT, &nchk}, {"nchk2", MMO_INT, &nchk2},
    {"dt", MMO_DBL, &dt}, {"t", MMO_DBL, &t},
    {"tautp", MMO_DBL, &tautp}, {"temp0", MMO_DBL, &temp0},
    {"tempi", MMO_DBL, &tempi}, {"vlimit", MMO_DBL, &vlimit},
    {"gamma_ln", MMO_DBL, &gamma_ln}, {"genmass", MMO_DBL, &genmass},
    {"wcons", MMO_DBL, &wcons}, {"ntpr_md", MMO_INT, &ntpr_md},
    {"zerov", MMO_INT, &zerov}, {"k4d", MMO_DBL, &k4d},
    {"ips", MMO_INT, &ips}, {"gb", MMO_INT, &gb},
    {"gb_debug", MMO_INT, &gb_debug}, {"nr_debug", MMO_INT, &nr_debug},
    {"gb2_debug", MMO_INT, &gb2_debug}, {"gbsa_debug", MMO_INT, &gbsa_debug},
    {"e_debug", MMO_INT, &e_debug}, {"epsext", MMO_DBL, &epsext},
    {"kappa", MMO_DBL, &kappa}, {"rgbmax", MMO_DBL, &rgbmax},
    {"surften", MMO_DBL, &surften}, {"dradius", MMO_DBL, &dradius},
    {"deltar", MMO_DBL, &deltar}, {"rwater", MMO_DBL, &rwater},
    {"alphanp", MMO_DBL, &alphanp}, {"kappanp", MMO_DBL, &kappanp},
    {"min_volume", MMO_DBL, &min_volume},
    {"max_set_size", MMO_INT, &max_set_size},
    {"MPI_min_tasks", MMO_INT, &MPI_min_tasks},
    {"cull_np_lists", MMO_INT, &cull_np_lists},
    {"use_lower_tri", MMO_INT, &use_lower_tri},
    {"dynamic_loops", MMO_INT, &dynamic_loops},
    {"blocksize", MMO_INT, &blocksize}, {"gbsa", MMO_INT, &gbsa},
    {"dim", MMO_INT, &dim}, {"diel", MMO_DIEL, &dield},
    {"dielc", MMO_DBL, &dielc}, {"rattle", MMO_INT, &irattle},
  };
  size_t i;
  for (i = 0; i < sizeof(table) / sizeof(table[0]); i++) {
    if (strcmp(table[i].key, key) == 0) {
      *kind = table[i].kind;
      *addr = table[i].addr;
      return 1;
    }
  }
  return 0;
}

int mm_options(char *opts)
{
  const char *p = opts;
  char key[64], val[128];
  while (*p) {
    const char *start, *vs;
    size_t kl, vl;
    int kind;
    void *addr;
    while (*p == ' ' || *p == ',' || *p == '\t' || *p == '\n')
      p++;
    if (!*p)
      break;
    start = p;
    while (isalnum((unsigned char)*p) || *p == '_')
      p++;
    kl = (size_t)(p - start);
    if (kl == 0 || kl >= sizeof(key)) {
      fprintf(stderr, "Error: mm_option: unknown keyword or invalid value: %s\n", start);
      exit(1);
    }
    memcpy(key, start, kl);
    key[kl] = '\0';
    while (*p == ' ')
      p++;
    if (*p == '=') {
      p++;
      while (*p == ' ')
        p++;
    }
    vs = p;
    while (*p && *p != ' ' && *p != ',' && *p != '\t' && *p != '\n')
      p++;
    vl = (size_t)(p - vs);
    if (vl == 0 || vl >= sizeof(val) || !mmo_lookup(key, &kind, &addr)) {
      fprintf(stderr, "Error: mm_option: unknown keyword or invalid value: %s\n", key);
      exit(1);
    }
    memcpy(val, vs, vl);
    val[vl] = '\0';
    if (mytaskid == 0)
      fprintf(nabout, "\tmm_options:  %.*s\n", (int)(p - start), start);
    if (kind == MMO_DBL) {
      *(double *)addr = atof(val);
    } else if (kind == MMO_INT) {
      *(int *)addr = atoi(val);
      if ((strcmp(key, "ntpr") == 0 || strcmp(key, "ntpr_md") == 0) &&
          *(int *)addr == 0)
        *(int *)addr = 9999999;
    } else {
      if (strcmp(val, "Yammp") == 0) dield = -5;
      else if (strcmp(val, "R94") == 0) dield = -4;
      else if (strcmp(val, "RL94") == 0) dield = -3;
      else if (strcmp(val, "RL") == 0) dield = -2;
      else if (strcmp(val, "R") == 0) dield = 0;
      else if (strcmp(val, "C") == 0) dield = 1;
      else {
        fprintf(stderr, "Error: mm_option: unknown keyword or invalid value: %s\n", val);
        exit(1);
      }
    }
  }
  return 0;
}
