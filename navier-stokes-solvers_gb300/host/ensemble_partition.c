/*
 * Partition of ensemble members over ranks (one GPU per rank).
 *
 * No reference counterpart: the reference advances one solver per call and has
 * no distributed code.  Ensemble members are independent solvers, so they are
 * the natural unit to spread over GPUs; a single field would need an
 * all-to-all transpose per 2-D transform and is not split.
 *
 * Longest processing time first (Graham 1969): members sorted by cost
 * n^2 log2(n^2) in decreasing order (ties: lower member index first) go one at
 * a time to the rank with the smallest total cost so far (ties: lower rank).
 * The result is a pure function of the member list and the rank count, so
 * every rank computes the same partition locally and no exchange is needed;
 * the only cross-rank traffic of an ensemble run is the gather of per-member
 * diagnostics.  LPT's makespan is within 4/3 of the optimum.
 */
#include <math.h>
#include <stdlib.h>

#include "ns_gpu.h"

typedef struct {
    double cost;
    int member;
} ns_part_item;

static int ns_part_cmp(const void *a, const void *b) {
    const ns_part_item *x = (const ns_part_item *)a, *y = (const ns_part_item *)b;
    if (x->cost > y->cost) return -1;
    if (x->cost < y->cost) return 1;
    return x->member - y->member;
}

double ns_ensemble_member_cost(int n) {
    if (n < 2) return 0.0;
    const double pts = (double)n * (double)n;
    return pts * log2(pts);
}

int ns_ensemble_partition(int nmembers, const int *n, int nranks, int *rank_of_member, double *rank_cost) {
    if (nmembers < 0 || nranks < 1 || (nmembers > 0 && (!n || !rank_of_member))) return NS_GPU_ERR_INVALID;
    for (int m = 0; m < nmembers; ++m)
        if (n[m] < 2) return NS_GPU_ERR_INVALID;
    ns_part_item *items = (ns_part_item *)malloc(sizeof(ns_part_item) * (size_t)(nmembers > 0 ? nmembers : 1));
    double *load = (double *)calloc((size_t)nranks, sizeof(double));
    if (!items || !load) {
        free(items);
        free(load);
        return NS_GPU_ERR_ALLOC;
    }
    for (int m = 0; m < nmembers; ++m) {
        items[m].cost = ns_ensemble_member_cost(n[m]);
        items[m].member = m;
    }
    qsort(items, (size_t)nmembers, sizeof(ns_part_item), ns_part_cmp);
    for (int i = 0; i < nmembers; ++i) {
        int best = 0;
        for (int r = 1; r < nranks; ++r)
            if (load[r] < load[best]) best = r;
        load[best] += items[i].cost;
        rank_of_member[items[i].member] = best;
    }
    if (rank_cost)
        for (int r = 0; r < nranks; ++r) rank_cost[r] = load[r];
    free(items);
    free(load);
    return NS_GPU_OK;
}
