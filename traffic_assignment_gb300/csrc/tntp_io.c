/*
 * tntp_io.c - TNTP text formats and host-side helpers of the drop-in C ABI.
 *
 * Same signatures, formats and error behaviour as the reference's
 * tap/parsetapfiles.c and the host-only parts of tap/tap_functions.c and
 * tap/sssp_pape.c: network, trips, flows, net-mods and trip-mods parsers, the
 * flows printer, the forward-star builder, demand bookkeeping and trip
 * modifications.  These are input/output conversions; every link-array
 * computation of the solver runs on the GPU (capi.cpp, linkops.cu).
 */
#define _GNU_SOURCE
#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "tap_gpu.h"

#define LINE_MAX_LEN 65536

static int blank_or_comment(const char *s)
{
  if (s[0] == '~') return 1;
  for (; *s; ++s)
    if (!isspace((unsigned char)*s)) return 0;
  return 1;
}

/* value of a "<TAG> value" metadata line, or NULL when the tag is unclosed */
static const char *meta_value(const char *line)
{
  const char *close = strchr(line, '>');
  if (!close) return NULL;
  return close + 1;
}

static int tag_is(const char *line, const char *tag) { return strncmp(line, tag, strlen(tag)) == 0; }

/* tap/parsetapfiles.c:62-146 */
int parse_net_file(FILE *fp, net_data_t *net)
{
  char *buf = malloc(LINE_MAX_LEN);
  long cap = 1024, count = 0;
  if (!buf) return -1;
  net->num_zones = net->num_nodes = net->num_links = 0;
  net->first_thru_node = 1;
  net->links = malloc(sizeof(link_data_t) * cap);
  if (!net->links) { free(buf); return -1; }
  while (fgets(buf, LINE_MAX_LEN, fp)) {
    if (blank_or_comment(buf)) continue;
    if (buf[0] == '<') {
      const char *v = meta_value(buf);
      if (!v) {
        fprintf(stderr, "error: no closing '>' on metadata tag: %s\n", buf);
        free(buf);
        return -1;
      }
      if (tag_is(buf, "<NUMBER OF ZONES>")) net->num_zones = atol(v);
      else if (tag_is(buf, "<NUMBER OF NODES>")) net->num_nodes = atol(v);
      else if (tag_is(buf, "<FIRST THRU NODE>")) net->first_thru_node = atol(v);
      else if (tag_is(buf, "<NUMBER OF LINKS>")) net->num_links = atol(v);
      else if (!tag_is(buf, "<END OF METADATA>"))
        fprintf(stderr, "warning: unknown metadata tag: %s\n", buf);
      continue;
    }
    if (count == cap) {
      link_data_t *n = realloc(net->links, sizeof(link_data_t) * cap * 2);
      if (!n) { free(buf); return -1; }
      net->links = n;
      cap *= 2;
    }
    char *save = NULL, *tok[10];
    int nt = 0;
    for (char *t = strtok_r(buf, " \t\r\n", &save); t && nt < 10; t = strtok_r(NULL, " \t\r\n", &save))
      tok[nt++] = t;
    if (nt < 10) {
      fprintf(stderr, "error: short link line %ld in net file\n", count + 1);
      free(buf);
      return -1;
    }
    link_data_t *l = &net->links[count++];
    l->init_node = atol(tok[0]);
    l->term_node = atol(tok[1]);
    l->capacity = atof(tok[2]);
    l->length = atof(tok[3]);
    l->free_flow_time = atof(tok[4]);
    l->B = atof(tok[5]);
    l->power = atof(tok[6]);
    l->speed_limit = atof(tok[7]);
    l->toll = atof(tok[8]);
    l->link_type = (short)atoi(tok[9]);
  }
  free(buf);
  if (count != net->num_links) {
    fprintf(stderr, "error: num_links %ld but %ld links\n", net->num_links, count);
    return -1;
  }
  return 0;
}

typedef struct {
  demand_data_t *v;
  long n, cap;
} dlist_t;

static int dlist_push(dlist_t *l, long dest, double dem)
{
  if (l->n + 1 >= l->cap) {
    long nc = l->cap ? l->cap * 2 : 16;
    demand_data_t *nv = realloc(l->v, sizeof(demand_data_t) * nc);
    if (!nv) return -1;
    l->v = nv;
    l->cap = nc;
  }
  l->v[l->n].dest = dest;
  l->v[l->n].demand = dem;
  l->n++;
  l->v[l->n].dest = 0; /* terminator */
  l->v[l->n].demand = 0;
  return 0;
}

/* tap/parsetapfiles.c:181-311 */
int parse_trips_file(FILE *fp, demand_data_t **demands[], long *num_zones)
{
  char *buf = malloc(LINE_MAX_LEN);
  dlist_t *lists = NULL;
  long zones = 0, cur = -1;
  double total_od = 0, total = 0;
  int rc = -1;
  if (!buf) return -1;
  *demands = NULL;
  *num_zones = 0;
  while (fgets(buf, LINE_MAX_LEN, fp)) {
    if (blank_or_comment(buf)) continue;
    if (buf[0] == '<') {
      const char *v = meta_value(buf);
      if (!v) {
        fprintf(stderr, "error: no closing '>' on metadata tag: %s\n", buf);
        goto out;
      }
      if (tag_is(buf, "<NUMBER OF ZONES>")) zones = atol(v);
      else if (tag_is(buf, "<TOTAL OD FLOW>")) total_od = atof(v);
      else if (tag_is(buf, "<END OF METADATA>")) {
        if (!lists) {
          lists = calloc((size_t)zones + 1, sizeof(dlist_t));
          if (!lists) goto out;
        }
      } else
        fprintf(stderr, "warning: unknown metadata tag: %s\n", buf);
      continue;
    }
    if (!lists) {
      lists = calloc((size_t)zones + 1, sizeof(dlist_t));
      if (!lists) goto out;
    }
    if (strncmp(buf, "Origin", 6) == 0) {
      if (sscanf(buf, "Origin %ld", &cur) != 1) {
        fprintf(stderr, "error parsing origin: %s\n", buf);
        goto out;
      }
      if (cur < 1 || cur > zones) {
        fprintf(stderr, "error: origin %ld outside 1..%ld\n", cur, zones);
        goto out;
      }
      if (lists[cur].v) {
        fprintf(stderr, "error: multiple entries for Origin %ld\n", cur);
        goto out;
      }
      lists[cur].v = calloc(16, sizeof(demand_data_t));
      lists[cur].cap = 16;
      if (!lists[cur].v) goto out;
      continue;
    }
    if (cur < 1) continue;
    char *save = NULL;
    for (char *item = strtok_r(buf, ";", &save); item; item = strtok_r(NULL, ";", &save)) {
      char *colon = strchr(item, ':');
      if (!colon) continue;
      *colon = '\0';
      long dest = atol(item);
      double dem = atof(colon + 1);
      if (dest > zones) fprintf(stderr, "warning: dest %ld > num_zones %ld\n", dest, zones);
      if (dlist_push(&lists[cur], dest, dem) != 0) goto out;
      total += dem;
    }
  }
  if (!lists) {
    lists = calloc((size_t)zones + 1, sizeof(dlist_t));
    if (!lists) goto out;
  }
  *demands = calloc((size_t)zones + 1, sizeof(demand_data_t *));
  if (!*demands) goto out;
  for (long o = 1; o <= zones; ++o) {
    if (!lists[o].v) {
      fprintf(stderr, "warning: no trip data for origin %ld\n", o);
      lists[o].v = calloc(1, sizeof(demand_data_t));
      if (!lists[o].v) goto out;
    }
    (*demands)[o] = lists[o].v;
    lists[o].v = NULL;
  }
  if (fabs(total_od - total) > 1e-08)
    fprintf(stderr, "warning: total_od_flow %f != %f\n", total_od, total);
  *num_zones = zones;
  rc = 0;
out:
  if (lists) {
    for (long o = 0; o <= zones; ++o) free(lists[o].v);
    free(lists);
  }
  free(buf);
  return rc;
}

/* tap/parsetapfiles.c:344-423 */
int parse_flows_file(FILE *flow_fp, link_flow_t **link_flows, long *num_links)
{
  char *buf = malloc(LINE_MAX_LEN);
  long cap = 1024, count = 0, meta_links = 0;
  if (!buf) return -1;
  *link_flows = malloc(sizeof(link_flow_t) * cap);
  if (!*link_flows) { free(buf); return -1; }
  while (fgets(buf, LINE_MAX_LEN, flow_fp)) {
    if (blank_or_comment(buf)) continue;
    if (buf[0] == '<') {
      const char *v = meta_value(buf);
      if (!v) {
        fprintf(stderr, "error: no closing '>' on metadata tag: %s\n", buf);
        free(buf);
        return -1;
      }
      if (tag_is(buf, "<NUMBER OF LINKS>")) meta_links = atol(v);
      else if (!tag_is(buf, "<NUMBER OF NODES>") && !tag_is(buf, "<END OF METADATA>"))
        fprintf(stderr, "warning: unknown metadata tag: %s\n", buf);
      continue;
    }
    if (count == cap) {
      link_flow_t *n = realloc(*link_flows, sizeof(link_flow_t) * cap * 2);
      if (!n) { free(buf); return -1; }
      *link_flows = n;
      cap *= 2;
    }
    char *save = NULL, *tok[5];
    int nt = 0;
    for (char *t = strtok_r(buf, "\t;\r\n", &save); t && nt < 5; t = strtok_r(NULL, "\t;\r\n", &save))
      tok[nt++] = t;
    if (nt < 5 || strchr(tok[2], ':') == NULL) {
      fprintf(stderr, "bad line in flows file: %s\n", buf);
      free(buf);
      return -1;
    }
    link_flow_t *f = &(*link_flows)[count++];
    f->init_node = atol(tok[0]);
    f->term_node = atol(tok[1]);
    f->volume = atof(tok[3]);
    f->cost = atof(tok[4]);
  }
  free(buf);
  if (count != meta_links) {
    fprintf(stderr, "error: num_links %ld but %ld links\n", meta_links, count);
    return -1;
  }
  *num_links = count;
  return 0;
}

/* tap/parsetapfiles.c:457-516 */
int parse_net_mod_file(FILE *fp, net_mod_t **mods, int *num_mods)
{
  char *buf = malloc(LINE_MAX_LEN);
  long cap = 16, count = 0;
  if (!buf) return -1;
  *mods = malloc(sizeof(net_mod_t) * cap);
  if (!*mods) { free(buf); return -1; }
  while (fgets(buf, LINE_MAX_LEN, fp)) {
    if (blank_or_comment(buf)) continue;
    if (count == cap) {
      net_mod_t *n = realloc(*mods, sizeof(net_mod_t) * cap * 2);
      if (!n) { free(buf); return -1; }
      *mods = n;
      cap *= 2;
    }
    char *save = NULL, *tok[13];
    int nt = 0;
    for (char *t = strtok_r(buf, "\t\r\n", &save); t && nt < 13; t = strtok_r(NULL, "\t\r\n", &save))
      tok[nt++] = t;
    if (nt < 12) {
      fprintf(stderr, "error: short line in net mods file\n");
      free(buf);
      return -1;
    }
    net_mod_t *m = &(*mods)[count];
    memset(m, 0, sizeof(*m));
    strncpy(m->change_id, tok[0], MAX_CHANGE_ID_LEN);
    if (strcmp(tok[1], "ADD") == 0) m->modtype = MOD_TYPE_ADD_E;
    else if (strcmp(tok[1], "CHANGE") == 0) m->modtype = MOD_TYPE_CHANGE_E;
    else {
      fprintf(stderr, "invalid change type '%s'\n", tok[1]);
      free(buf);
      return -1;
    }
    link_data_t *l = &m->mod_link;
    l->init_node = atol(tok[2]);
    l->term_node = atol(tok[3]);
    l->capacity = atof(tok[4]);
    l->length = atof(tok[5]);
    l->free_flow_time = atof(tok[6]);
    l->B = atof(tok[7]);
    l->power = atof(tok[8]);
    l->speed_limit = atof(tok[9]);
    l->toll = atof(tok[10]);
    l->link_type = (short)atoi(tok[11]);
    m->project_cost = nt > 12 ? atof(tok[12]) : 0.0;
    count++;
  }
  free(buf);
  *num_mods = (int)count;
  return 0;
}

/* tap/parsetapfiles.c:528-540 */
int link_data_compar(const void *a, const void *b)
{
  const link_data_t *x = a, *y = b;
  if (x->init_node != y->init_node) return x->init_node < y->init_node ? -1 : 1;
  if (x->term_node != y->term_node) return x->term_node < y->term_node ? -1 : 1;
  return 0;
}

/* tap/tap_functions.c:274-286 */
int adjlist_entry_compar(const void *a, const void *b) { return link_data_compar(a, b); }

/* tap/parsetapfiles.c:573-638 */
int parse_trip_mod_file(FILE *fp, trip_mod_t **mods, int *num_mods)
{
  char *buf = malloc(LINE_MAX_LEN);
  long cap = 16, count = 0;
  if (!buf) return -1;
  *mods = malloc(sizeof(trip_mod_t) * cap);
  if (!*mods) { free(buf); return -1; }
  while (fgets(buf, LINE_MAX_LEN, fp)) {
    if (blank_or_comment(buf)) continue;
    if (count == cap) {
      trip_mod_t *n = realloc(*mods, sizeof(trip_mod_t) * cap * 2);
      if (!n) { free(buf); return -1; }
      *mods = n;
      cap *= 2;
    }
    char *save = NULL, *tok[5];
    int nt = 0;
    for (char *t = strtok_r(buf, "\t\r\n", &save); t && nt < 5; t = strtok_r(NULL, "\t\r\n", &save))
      tok[nt++] = t;
    if (nt < 5) {
      fprintf(stderr, "error: short line in trip mods file\n");
      free(buf);
      return -1;
    }
    trip_mod_t *m = &(*mods)[count];
    memset(m, 0, sizeof(*m));
    strncpy(m->trip_change_id, tok[0], MAX_CHANGE_ID_LEN);
    if (strcmp(tok[1], "P2P") == 0) m->trip_modtype = TRIP_MOD_TYPE_POINT_E;
    else if (strcmp(tok[1], "UNIFORM") == 0) m->trip_modtype = TRIP_MOD_TYPE_UNIFORM_E;
    else if (strcmp(tok[1], "ALL") == 0) m->trip_modtype = TRIP_MOD_TYPE_ALL_E;
    else {
      fprintf(stderr, "invalid trip data change type '%s'\n", tok[1]);
      free(buf);
      return -1;
    }
    m->origin = atol(tok[2]);
    m->dest = atol(tok[3]);
    m->multiplier = atof(tok[4]);
    if (m->trip_modtype == TRIP_MOD_TYPE_POINT_E && (m->origin == 0 || m->dest == 0)) {
      fprintf(stderr, "ERROR: origin and dest must be nonzero for point-to-point\n");
      free(buf);
      return -1;
    }
    if (m->trip_modtype != TRIP_MOD_TYPE_ALL_E && m->origin == 0 && m->dest == 0) {
      fprintf(stderr, "ERROR: cannot have 0 for both origin and dest except type ALL\n");
      free(buf);
      return -1;
    }
    count++;
  }
  free(buf);
  *num_mods = (int)count;
  return 0;
}

/* tap/tap_functions.c:431-445 */
void print_flow(FILE *fp, const net_data_t *net, const double link_volumes[],
                const double link_costs[])
{
  fprintf(fp, "<NUMBER OF NODES>\t%ld\n", net->num_nodes);
  fprintf(fp, "<NUMBER OF LINKS>\t%ld\n", net->num_links);
  fprintf(fp, "<END OF METADATA>\n");
  fprintf(fp, "\n");
  fprintf(fp, "~\tTail\tHead\t:\tVolume\tCost\t;\n");
  for (long k = 0; k < net->num_links; k++)
    fprintf(fp, "\t%ld\t%ld\t:\t%.15f\t%.15f;\n", net->links[k].init_node,
            net->links[k].term_node, link_volumes[k], link_costs[k]);
}

/* tap/tap_functions.c:377-386: origins 1..num_zones-1 (callers pass Z+1) */
double demand_sum(demand_data_t *const demands[], long num_zones)
{
  double s = 0;
  for (long o = 1; o < num_zones; o++)
    for (long i = 0; demands[o][i].dest != 0; i++) s += demands[o][i].demand;
  return s;
}

/* tap/tap_functions.c:313-339 (links must already be sorted by (init, term)) */
void adjlist_to_packed_arrays(link_data_t adjlist[], long num_nodes, long num_edges, long Va[],
                              long Ea[], double Wa[])
{
  long e = 0;
  for (long v = 0; v < num_nodes; v++) {
    Va[v] = e;
    while (e < num_edges && adjlist[e].init_node == v) {
      Ea[e] = adjlist[e].term_node;
      Wa[e] = adjlist[e].free_flow_time;
      e++;
    }
    if (v != 0 && Va[v] == e) fprintf(stderr, "warning: node %ld has no links out\n", v);
  }
  Va[num_nodes] = e;
}

/* tap/tap_functions.c:55-65 (one link, host scalar) */
double bpr_cost_function(const link_data_t *link, double Q)
{
  return link->free_flow_time * (1.0 + link->B * pow(Q / link->capacity, link->power));
}

/* tap/tap_functions.c:112-126 (one link, host scalar) */
double linkcost_integral(const link_data_t *link, double Q)
{
  if (link->power >= 0)
    return Q * link->free_flow_time *
           (1 + ((link->B / pow(link->capacity, link->power)) / (link->power + 1)) *
                    pow(Q, link->power));
  return 0;
}

/* tap/sssp_pape.c:237-253: walk a predecessor-node array back from dest */
void get_shortest_path(long pred[], long orig, long dest, long path[], long *pathlen)
{
  long v = dest;
  *pathlen = 0;
  if (pred[v] == -1) return;
  while (v != orig) {
    path[(*pathlen)++] = v;
    v = pred[v];
    if (v < 0) return;
  }
  path[(*pathlen)++] = orig;
}

/* tap/tap_functions.c:521-598 */
int apply_trip_modification(demand_data_t *demands[], trip_mod_t *mod, long num_zones)
{
  if (mod->origin > num_zones || mod->dest > num_zones || mod->origin < 0 || mod->dest < 0) {
    fprintf(stderr, "ERROR: bad origin %ld or dest %ld in trip modification\n", mod->origin,
            mod->dest);
    return -1;
  }
  switch (mod->trip_modtype) {
    case TRIP_MOD_TYPE_POINT_E:
      fprintf(stderr, "[tripchange %s] %ld -> %ld multiplier %f\n", mod->trip_change_id,
              mod->origin, mod->dest, mod->multiplier);
      for (long i = 0; demands[mod->origin][i].dest != 0; i++)
        if (demands[mod->origin][i].dest == mod->dest) {
          demands[mod->origin][i].demand *= mod->multiplier;
          break;
        }
      return 0;
    case TRIP_MOD_TYPE_UNIFORM_E:
      if (mod->dest == 0 && mod->origin > 0) {
        fprintf(stderr, "[tripchange %s] origin %ld multiplier %f\n", mod->trip_change_id,
                mod->origin, mod->multiplier);
        for (long i = 0; demands[mod->origin][i].dest != 0; i++)
          demands[mod->origin][i].demand *= mod->multiplier;
        return 0;
      }
      if (mod->origin == 0 && mod->dest > 0) {
        fprintf(stderr, "[tripchange %s] dest %ld multiplier %f\n", mod->trip_change_id,
                mod->dest, mod->multiplier);
        for (long o = 1; o <= num_zones; o++)
          for (long j = 0; demands[o][j].dest != 0; j++)
            if (demands[o][j].dest == mod->dest) demands[o][j].demand *= mod->multiplier;
        return 0;
      }
      fprintf(stderr, "ERROR: both origin and dest nonzero in uniform trip mod\n");
      return -1;
    case TRIP_MOD_TYPE_ALL_E:
      fprintf(stderr, "[tripchange %s] ALL multiplier %f\n", mod->trip_change_id, mod->multiplier);
      for (long o = 1; o <= num_zones; o++)
        for (long j = 0; demands[o][j].dest != 0; j++) demands[o][j].demand *= mod->multiplier;
      return 0;
    default:
      fprintf(stderr, "bad trip modification type %d\n", mod->trip_modtype);
      return -1;
  }
}
