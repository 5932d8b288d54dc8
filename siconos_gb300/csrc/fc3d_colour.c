/* Kempe-chain reduction of a contact colouring (host code).
 *
 * Two contacts conflict when they share a body, i.e. when W holds a block
 * between them; the conflict graph of a friction-contact problem is the
 * line graph of the body graph.  Greedy vertex colourings of such graphs
 * (graph_tools.c:592-940 in the reference, the device Jones-Plassmann
 * colouring here) end with a few more colours than needed: a cubic sphere
 * lattice, whose body graph is bipartite with degree 6, is 6-edge-colourable
 * (Konig's theorem) but greedy stops at 8, the last class nearly empty.
 * Every colour costs the Gauss-Seidel sweep one ordered phase, so fewer
 * colours make a faster sweep.
 *
 * The reduction empties the highest class one contact at a time.  A contact
 * v takes the smallest colour none of its neighbours has; when there is
 * none, it looks for colours a, b such that the (a, b)-Kempe components
 * through v's a-coloured neighbours hold none of v's b-coloured neighbours:
 * exchanging a and b on those components keeps the colouring proper and
 * frees a for v (the alternating-path step of the edge-colouring proof,
 * which always succeeds on bipartite body graphs while the classes left
 * are at least the largest number of contacts of one body).  A class that
 * cannot be emptied stays; the result is a proper colouring in any case.
 *
 * The outcome depends only on the graph and the input colouring, not on the
 * order of the adjacency lists: candidates are taken in index order, colour
 * pairs in a fixed order, and a Kempe component is exchanged whole. */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define COLOUR_MAX 128

static int has_colour(const uint64_t m[2], int c) { return (int)((m[c >> 6] >> (c & 63)) & 1u); }

/* gptr/adj: the conflict graph, symmetric CSR (duplicates allowed), nc
 * vertices; colour[nc] a proper colouring with ncol colours.  work_cap
 * bounds the vertices one Kempe search visits (<= 0: nc).  Returns the new
 * number of colours, or a negative value when memory runs out (colour then
 * still proper). */
int fc3dgpu_colour_reduce(int nc, const int *gptr, const int *adj, int *colour, int ncol, int work_cap) {
  if (nc <= 0 || ncol <= 1 || ncol > COLOUR_MAX) return ncol;
  if (work_cap <= 0) work_cap = nc;
  int *seen = (int *)calloc((size_t)nc, sizeof(int));
  int *nbr = (int *)calloc((size_t)nc, sizeof(int));
  int *queue = (int *)malloc(sizeof(int) * (size_t)nc);
  int *cls = (int *)malloc(sizeof(int) * (size_t)nc);
  if (!seen || !nbr || !queue || !cls) {
    free(seen);
    free(nbr);
    free(queue);
    free(cls);
    return -1;
  }
  int gen = 0, ngen = 0;
  while (ncol > 1) {
    const int top = ncol - 1;
    int n = 0;
    for (int v = 0; v < nc; v++)
      if (colour[v] == top) cls[n++] = v;
    int left = 0;
    for (int t = 0; t < n; t++) {
      const int v = cls[t];
      uint64_t used[2] = {0, 0};
      ngen++;
      for (int k = gptr[v]; k < gptr[v + 1]; k++) {
        const int w = adj[k];
        if (w == v) continue;
        used[colour[w] >> 6] |= 1ull << (colour[w] & 63);
        nbr[w] = ngen;
      }
      int c = -1;
      for (int x = 0; x < top && c < 0; x++)
        if (!has_colour(used, x)) c = x;
      for (int a = 0; a < top && c < 0; a++) {
        for (int b = 0; b < top && c < 0; b++) {
          if (b == a || !has_colour(used, b)) continue;
          /* the (a, b) components through v's a-neighbours */
          gen++;
          int qn = 0, ok = 1;
          for (int k = gptr[v]; k < gptr[v + 1]; k++) {
            const int w = adj[k];
            if (w != v && colour[w] == a && seen[w] != gen) {
              seen[w] = gen;
              queue[qn++] = w;
            }
          }
          for (int h = 0; h < qn && ok; h++) {
            const int u = queue[h];
            for (int k = gptr[u]; k < gptr[u + 1]; k++) {
              const int w = adj[k];
              if (seen[w] == gen || (colour[w] != a && colour[w] != b)) continue;
              if (colour[w] == b && nbr[w] == ngen) {
                ok = 0;  /* a b-neighbour of v would turn a */
                break;
              }
              if (qn >= work_cap) {
                ok = 0;
                break;
              }
              seen[w] = gen;
              queue[qn++] = w;
            }
          }
          if (!ok) continue;
          for (int h = 0; h < qn; h++) colour[queue[h]] = colour[queue[h]] == a ? b : a;
          c = a;
        }
      }
      if (c >= 0)
        colour[v] = c;
      else
        left++;
    }
    if (left) break;
    ncol = top;
  }
  free(seen);
  free(nbr);
  free(queue);
  free(cls);
  return ncol;
}
