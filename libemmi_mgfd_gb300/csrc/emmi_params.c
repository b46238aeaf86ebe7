/* SU-style key=value parameters, compatible with the reference's getpar
 * (src/cstd.c:836-1569): arguments key=value, the last occurrence wins, a
 * par=file argument adds the file's key=value tokens, vectors are comma
 * separated.  The drop-in GPU library reads its solver knobs through these
 * functions when the host program links this file. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define EH_MAXARGS 4096
static char *g_args[EH_MAXARGS];
static int g_nargs = 0;

static void add_arg(const char *a) {
  if (g_nargs < EH_MAXARGS && strchr(a, '=')) g_args[g_nargs++] = strdup(a);
}

static void add_parfile(const char *path) {
  FILE *fp = fopen(path, "r");
  if (!fp) {
    fprintf(stderr, "cannot open par file %s\n", path);
    exit(1);
  }
  char tok[4096];
  while (fscanf(fp, "%4095s", tok) == 1) {
    if (tok[0] == '#') { /* comment to end of line */
      int c;
      while ((c = fgetc(fp)) != EOF && c != '\n') {
      }
      continue;
    }
    add_arg(tok);
  }
  fclose(fp);
}

void initargs(int argc, char **argv) {
  g_nargs = 0;
  for (int i = 1; i < argc; i++) {
    if (strncmp(argv[i], "par=", 4) == 0)
      add_parfile(argv[i] + 4);
    else
      add_arg(argv[i]);
  }
}

/* value string of the last occurrence of name, or NULL */
static const char *lookup(const char *name) {
  const size_t n = strlen(name);
  for (int i = g_nargs - 1; i >= 0; i--)
    if (strncmp(g_args[i], name, n) == 0 && g_args[i][n] == '=') return g_args[i] + n + 1;
  return NULL;
}

int countparval(const char *name) {
  const char *v = lookup(name);
  if (!v || !*v) return 0;
  int c = 1;
  for (const char *p = v; *p; p++)
    if (*p == ',') c++;
  return c;
}

int getparint(char *name, int *p) {
  const char *v = lookup(name);
  if (!v) return 0;
  char *end;
  *p = (int)strtol(v, &end, 10);
  if (end == v) {
    fprintf(stderr, "bad integer for %s: %s\n", name, v);
    exit(1);
  }
  return 1;
}

int getpardouble(char *name, double *p) {
  const char *v = lookup(name);
  if (!v) return 0;
  char *end;
  *p = strtod(v, &end);
  if (end == v) {
    fprintf(stderr, "bad number for %s: %s\n", name, v);
    exit(1);
  }
  return 1;
}

/* float vector: fills as many comma-separated values as present */
int getparfloat(char *name, float *p) {
  const char *v = lookup(name);
  if (!v) return 0;
  int k = 0;
  const char *s = v;
  while (*s) {
    char *end;
    p[k++] = strtof(s, &end);
    if (end == s) {
      fprintf(stderr, "bad number for %s: %s\n", name, v);
      exit(1);
    }
    s = (*end == ',') ? end + 1 : end;
    if (*end != ',') break;
  }
  return k;
}

int getparstring(char *name, char **p) {
  const char *v = lookup(name);
  if (!v) return 0;
  *p = strdup(v);
  return 1;
}

int getparstringarray(char *name, char **p) {
  const char *v = lookup(name);
  if (!v) return 0;
  char *copy = strdup(v);
  int k = 0;
  for (char *t = strtok(copy, ","); t; t = strtok(NULL, ",")) p[k++] = t;
  return k;
}
