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
 * are at least the largest number of contacts of one body).  The first
 * contact of a class that cannot move ends the reduction (that class
 * stays); the result is a proper colouring in any case.
 *
 * The outcome depends only on the graph and the input colouring, not on the
 * order of the adjacency lists: candidates are taken in index order, colour
 * pairs in an order set by the colours around the candidate and its
 * lowest-index neighbour, and a Kempe component is exchanged whole.
 *
 * Most of the time goes to the Kempe searches, and their components grow with
 * the lattice (on 60x60x30 a tenth of the exchanges move more than 64
 * contacts, a few more than 1,000).  Trying every pair with a small search
 * cap before any pair with a larger one prefers short components: 1.35x less
 * time than taking the first pair that works on the 60x60x30 lattice, 1.57x
 * on 80x80x40, with as good a colouring (548 against 550 colour-order sweeps
 * to an error of 1e-3 on 60x60x30). */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define COLOUR_MAX 128
/* Kempe searches by iterative deepening: the components a search may visit
 * start at SEARCH_CAP0 vertices and grow by SEARCH_CAP_GROWTH.  A search that
 * reaches the cap fails whatever the order it visits the component in, so
 * the outcome still does not depend on the adjacency lists' order. */
#define SEARCH_CAP0 32
#define SEARCH_CAP_GROWTH 4

static int has_colour(const uint64_t m[2], int c) { return (int)((m[c >> 6] >> (c & 63)) & 1u); }

/* Exchange colours a and b on the (a, b)-Kempe components through v's
 * a-coloured neighbours, unless one holds a b-coloured neighbour of v
 * (nbr[w] == ngen marks v's neighbours) or a search passes work_cap
 * vertices; returns 1 when exchanged (a is then free for v). */
static int kempe_exchange(int v, int a, int b, const int *gptr, const int *adj, int *colour, int *seen, int gen,
                          const int *nbr, int ngen, int *queue, int work_cap) {
  int qn = 0;
  for (int k = gptr[v]; k < gptr[v + 1]; k++) {
    const int w = adj[k];
    if (w != v && colour[w] == a && seen[w] != gen) {
      seen[w] = gen;
      queue[qn++] = w;
    }
  }
  for (int h = 0; h < qn; h++) {
    const int u = queue[h];
    for (int k = gptr[u]; k < gptr[u + 1]; k++) {
      const int w = adj[k];
      if (seen[w] == gen || (colour[w] != a && colour[w] != b)) continue;
      if (colour[w] == b && nbr[w] == ngen) return 0; /* a b-neighbour of v would turn a */
      if (qn >= work_cap) return 0;
      seen[w] = gen;
      queue[qn++] = w;
    }
  }
  for (int h = 0; h < qn; h++) colour[queue[h]] = colour[queue[h]] == a ? b : a;
  return 1;
}

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
  int *side = (int *)calloc((size_t)nc, sizeof(int));
  if (!seen || !nbr || !queue || !cls || !side) {
    free(seen);
    free(nbr);
    free(queue);
    free(cls);
    free(side);
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
      int cnt[COLOUR_MAX];
      for (int x = 0; x < top; x++) cnt[x] = 0;
      ngen++;
      for (int k = gptr[v]; k < gptr[v + 1]; k++) {
        const int w = adj[k];
        if (w == v || nbr[w] == ngen) continue;
        used[colour[w] >> 6] |= 1ull << (colour[w] & 63);
        nbr[w] = ngen;
        if (colour[w] < top) cnt[colour[w]]++;
      }
      int c = -1;
      for (int x = 0; x < top && c < 0; x++)
        if (!has_colour(used, x)) c = x;
      /* Colour pairs to try.  On a line graph v joins two bodies: the
       * neighbours through the body of its lowest-index neighbour w0 are w0
       * and w0's neighbours (one clique), the others go through the second
       * body.  A colour a held only on the second side and a colour b held
       * only on the first is the pair of the edge-colouring proof; those
       * pairs come first, then every pair of held colours. */
      int w0 = -1;
      if (c < 0)
        for (int k = gptr[v]; k < gptr[v + 1]; k++)
          if (adj[k] != v && (w0 < 0 || adj[k] < w0)) w0 = adj[k];
      uint64_t s0[2] = {0, 0}, s1[2] = {0, 0};
      if (w0 >= 0) {
        for (int k = gptr[w0]; k < gptr[w0 + 1]; k++) side[adj[k]] = ngen;
        side[w0] = ngen;
        for (int k = gptr[v]; k < gptr[v + 1]; k++) {
          const int w = adj[k];
          if (w == v) continue;
          uint64_t *m = (side[w] == ngen) ? s0 : s1;
          m[colour[w] >> 6] |= 1ull << (colour[w] & 63);
        }
      }
      /* Every pair first with its search capped at SEARCH_CAP0 vertices,
       * then with the cap times SEARCH_CAP_GROWTH, up to work_cap: a pair
       * with short Kempe components goes before the first pair that works. */
      for (int cap = SEARCH_CAP0; c < 0; cap *= SEARCH_CAP_GROWTH) {
        const int lim = cap < work_cap ? cap : work_cap;
        for (int phase = 0; phase < 2 && c < 0; phase++)
          for (int a = 0; a < top && c < 0; a++)
            for (int b = 0; b < top && c < 0; b++) {
              if (a == b || cnt[a] == 0 || cnt[b] == 0) continue;
              const int pref = has_colour(s1, a) && !has_colour(s0, a) && has_colour(s0, b) && !has_colour(s1, b);
              if (pref != (phase == 0)) continue;
              if (kempe_exchange(v, a, b, gptr, adj, colour, seen, ++gen, nbr, ngen, queue, lim)) c = a;
            }
        if (lim >= work_cap) break;
      }
      if (c < 0) {
        left = 1;  /* the class stays: stop at its first contact that cannot move */
        break;
      }
      colour[v] = c;
    }
    if (left) break;
    ncol = top;
  }
  free(seen);
  free(nbr);
  free(queue);
  free(cls);
  free(side);
  return ncol;
}

/* Batches: every group (one problem of a batch: rows group_off[g] ..
 * group_off[g + 1] - 1, whose conflicts stay inside the group) is reduced on
 * its own, as fc3dgpu_colour_reduce reduces it alone, by up to nthreads host
 * threads taking groups in turn; the groups are independent, so the result
 * does not depend on the threads. */
typedef struct {
  int ngroups;
  const int *group_off, *gptr, *adj;
  int *colour, *out;
  int next; /* next group to take (atomic) */
} reduce_groups_job;

static void *reduce_groups_worker(void *arg) {
  reduce_groups_job *J = (reduce_groups_job *)arg;
  int *lg = NULL, *la = NULL;
  size_t lg_cap = 0, la_cap = 0;
  for (;;) {
    const int g = __atomic_fetch_add(&J->next, 1, __ATOMIC_RELAXED);
    if (g >= J->ngroups) break;
    const int o0 = J->group_off[g], n = J->group_off[g + 1] - o0;
    if (n <= 0) {
      J->out[g] = 0;
      continue;
    }
    const int a0 = J->gptr[o0], na = J->gptr[o0 + n] - a0;
    if ((size_t)n + 1 > lg_cap || (size_t)(na > 0 ? na : 1) > la_cap) {
      free(lg);
      free(la);
      lg_cap = (size_t)n + 1 > lg_cap ? (size_t)n + 1 : lg_cap;
      la_cap = (size_t)(na > 0 ? na : 1) > la_cap ? (size_t)(na > 0 ? na : 1) : la_cap;
      lg = (int *)malloc(sizeof(int) * lg_cap);
      la = (int *)malloc(sizeof(int) * la_cap);
      if (!lg || !la) {
        J->out[g] = -1;
        lg_cap = la_cap = 0;
        continue;
      }
    }
    for (int k = 0; k <= n; k++) lg[k] = J->gptr[o0 + k] - a0;
    for (int k = 0; k < na; k++) la[k] = J->adj[a0 + k] - o0;
    int ng = 0;
    for (int k = 0; k < n; k++)
      if (J->colour[o0 + k] + 1 > ng) ng = J->colour[o0 + k] + 1;
    const int r = fc3dgpu_colour_reduce(n, lg, la, J->colour + o0, ng, 0);
    J->out[g] = r > 0 ? r : (r < 0 ? r : ng);
  }
  free(lg);
  free(la);
  return NULL;
}

int fc3dgpu_colour_reduce_groups(int ngroups, const int *group_off, const int *gptr, const int *adj, int *colour,
                                 int nthreads) {
  if (ngroups <= 0) return 0;
  int *out = (int *)calloc((size_t)ngroups, sizeof(int));
  if (!out) return -1;
  reduce_groups_job J = {ngroups, group_off, gptr, adj, colour, out, 0};
  if (nthreads < 1) nthreads = 1;
  if (nthreads > ngroups) nthreads = ngroups;
  if (nthreads > 64) nthreads = 64;
  pthread_t th[64];
  int started = 0;
  for (int t = 1; t < nthreads; t++)
    if (pthread_create(&th[started], NULL, reduce_groups_worker, &J) == 0) started++;
  reduce_groups_worker(&J);
  for (int t = 0; t < started; t++) pthread_join(th[t], NULL);
  int mx = 0, bad = 0;
  for (int g = 0; g < ngroups; g++) {
    if (out[g] < 0) bad = 1;
    if (out[g] > mx) mx = out[g];
  }
  free(out);
  return bad ? -1 : mx;
}
