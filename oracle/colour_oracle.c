/* Host greedy colouring of the contact conflict graph -- TEST INFRASTRUCTURE.
 *
 * The oracle for the device colouring kernel.  Two contacts conflict when W
 * holds a nonzero off-diagonal block between them (in either direction):
 * they share a body, which is the adjacency the reference's colour-parallel
 * NSGS builds from an SBM (tools/parallel/graph_tools.c:773-866).  The
 * reference colours with PETSc's greedy distance-1 colouring (graph_tools.c:
 * 876-928); PETSc is absent, so this file restates a deterministic greedy
 * colouring of its own:
 *
 *   visit contacts by decreasing priority (ties: smaller index first) and give
 *   each the smallest colour no already-coloured neighbour holds.
 *
 * Priority = key(contact) from oracle_colour_priority below: a 32-bit integer
 * hash of the contact index (kind 0) or the conflict degree with the hash as
 * tie-break (kind 1, largest degree first).  The device kernel colours in
 * Jones-Plassmann rounds with the same priorities; a vertex's colour depends
 * only on its higher-priority neighbours, so both give the same colours. */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* lowbias32 integer hash (C. Wellons' published constants) */
static uint32_t hash32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x;
}

/* 32-bit key; larger key = coloured earlier. kind 1 puts the degree (capped
 * at 255) in the top byte. */
uint32_t oracle_colour_priority(uint32_t index, int kind, uint32_t degree) {
  uint32_t h = hash32(index ^ 0x9e3779b9U);
  if (kind == 1) return ((degree > 255 ? 255U : degree) << 24) | (h >> 8);
  return h;
}

/* symmetric conflict graph without the diagonal, CSR */
static void conflict_graph(int nc, const int64_t *rowptr, const int64_t *colidx, int64_t **gptr_out,
                           int32_t **gadj_out) {
  int64_t *cnt = (int64_t *)calloc((size_t)nc + 1, sizeof(int64_t));
  for (int i = 0; i < nc; i++)
    for (int64_t k = rowptr[i]; k < rowptr[i + 1]; k++) {
      int64_t j = colidx[k];
      if (j == i) continue;
      cnt[i + 1]++;
      cnt[j + 1]++;
    }
  for (int i = 0; i < nc; i++) cnt[i + 1] += cnt[i];
  int32_t *adj = (int32_t *)malloc(sizeof(int32_t) * (size_t)(cnt[nc] ? cnt[nc] : 1));
  int64_t *fill = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nc > 0 ? nc : 1));
  memcpy(fill, cnt, sizeof(int64_t) * (size_t)nc);
  for (int i = 0; i < nc; i++)
    for (int64_t k = rowptr[i]; k < rowptr[i + 1]; k++) {
      int64_t j = colidx[k];
      if (j == i) continue;
      adj[fill[i]++] = (int32_t)j;
      adj[fill[j]++] = i;
    }
  free(fill);
  *gptr_out = cnt;
  *gadj_out = adj;
}

static uint32_t *g_key;
static int cmp_prio(const void *a, const void *b) {
  int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
  if (g_key[x] != g_key[y]) return g_key[x] > g_key[y] ? -1 : 1;
  return (x > y) - (x < y);
}

static int greedy_in_key_order(int nc, const int64_t *gp, const int32_t *ga, uint32_t *key, int32_t *ord,
                               int32_t *colour) {
  for (int i = 0; i < nc; i++) {
    ord[i] = i;
    colour[i] = -1;
  }
  g_key = key;
  qsort(ord, (size_t)nc, sizeof(int32_t), cmp_prio);
  int ncol = 0;
  uint8_t used[1024];
  for (int t = 0; t < nc; t++) {
    int i = ord[t];
    memset(used, 0, sizeof(used));
    for (int64_t k = gp[i]; k < gp[i + 1]; k++) {
      int c = colour[ga[k]];
      if (c >= 0 && c < 1024) used[c] = 1;
    }
    int c = 0;
    while (c < 1024 && used[c]) c++;
    colour[i] = c;
    if (c + 1 > ncol) ncol = c + 1;
  }
  return ncol;
}

/* Colours in colour[nc]; returns the number of colours.  Degree for kind 1
 * counts distinct conflicting contacts.  kind >> 8 = number of iterated
 * greedy passes (Culberson): recolour greedily with the current classes
 * visited as blocks in reverse order (highest colour first), the kind-0
 * hash (top byte dropped) ordering a class's members. */
int oracle_colour_greedy(int nc, const int64_t *rowptr, const int64_t *colidx, int kind, int32_t *colour) {
  const int passes = (kind >> 8) & 0xff;
  kind &= 0xff;
  int64_t *gp;
  int32_t *ga;
  conflict_graph(nc, rowptr, colidx, &gp, &ga);
  uint32_t *key = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(nc > 0 ? nc : 1));
  int32_t *ord = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nc > 0 ? nc : 1));
  /* distinct-neighbour degree: W's structure may list (i,j) and (j,i) */
  int32_t *mark = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nc > 0 ? nc : 1));
  for (int i = 0; i < nc; i++) mark[i] = -1;
  for (int i = 0; i < nc; i++) {
    uint32_t d = 0;
    for (int64_t k = gp[i]; k < gp[i + 1]; k++)
      if (mark[ga[k]] != i) {
        mark[ga[k]] = i;
        d++;
      }
    key[i] = oracle_colour_priority((uint32_t)i, kind, d);
  }
  int ncol = greedy_in_key_order(nc, gp, ga, key, ord, colour);
  for (int pass = 0; pass < passes; pass++) {
    for (int i = 0; i < nc; i++)
      key[i] = ((uint32_t)colour[i] << 24) | (oracle_colour_priority((uint32_t)i, 0, 0) >> 8);
    ncol = greedy_in_key_order(nc, gp, ga, key, ord, colour);
  }
  free(key);
  free(ord);
  free(mark);
  free(gp);
  free(ga);
  return ncol;
}

/* 0 when no two conflicting contacts share a colour, else 1 + the first
 * offending contact index. */
int oracle_colour_check(int nc, const int64_t *rowptr, const int64_t *colidx, const int32_t *colour) {
  for (int i = 0; i < nc; i++) {
    if (colour[i] < 0) return i + 1;
    for (int64_t k = rowptr[i]; k < rowptr[i + 1]; k++) {
      int64_t j = colidx[k];
      if (j != i && colour[j] == colour[i]) return i + 1;
    }
  }
  return 0;
}
