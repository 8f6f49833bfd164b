/*
 * oracle_bench.c -- times the CPU restatement of snn::step on the Brunel network
 * (TEST INFRASTRUCTURE ONLY: bench.py's cpu_baseline / --impl reference leg runs it).
 *
 * usage: oracle_bench N P STEPS SEED0 THREADS [WARMUP]
 *   Builds THREADS independent Brunel networks (seeds SEED0, SEED0+1, ...; the same model as
 *   samples/brunel.cpp:75-116 with weights scaled by 0.1/P), one per thread, runs WARMUP
 *   untimed steps, then times STEPS steps of all networks in parallel.  Prints one JSON line.
 */
#define _POSIX_C_SOURCE 200809L
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <time.h>

#include "spice_oracle.h"

typedef struct {
	long long N, steps, warmup;
	double p;
	unsigned seed;
	long long events, spikes;
	double build_s;
	spo_net* net;
	pthread_barrier_t* bar;
} job;

static double now(void) {
	struct timespec ts;
	clock_gettime(CLOCK_MONOTONIC, &ts);
	return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

/* The Brunel network: P = N/2 Poisson (20 Hz), E = 0.4 N and I = 0.1 N LIF, six
 * fixed_probability(p) projections, weights 2/N and -10/N scaled by 0.1/p, delay 15 dt. */
spo_net* brunel(long long N, double p, unsigned seed) {
	float dt = 1e-4f, delay = 15e-4f;
	uint32_t s = seed;
	spo_net* n = spo_net_create(dt, delay, &s, 1);
	float rate = 20.0f;
	int P = spo_add_population(n, SPO_POISSON, N / 2, &rate, 1);
	int E = spo_add_population(n, SPO_LIF, N * 4 / 10, NULL, 0);
	int I = spo_add_population(n, SPO_LIF, N / 10, NULL, 0);
	float we = (float)((2.0 / N) * (0.1 / p)), wi = (float)((-10.0 / N) * (0.1 / p));
	spo_connect(n, P, E, p, delay, 0, we);
	spo_connect(n, P, I, p, delay, 0, we);
	spo_connect(n, E, E, p, delay, 0, we);
	spo_connect(n, E, I, p, delay, 0, we);
	spo_connect(n, I, E, p, delay, 0, wi);
	spo_connect(n, I, I, p, delay, 0, wi);
	return n;
}

static void* worker(void* arg) {
	job* j      = (job*)arg;
	double t0   = now();
	j->net      = brunel(j->N, j->p, j->seed);
	j->build_s  = now() - t0;
	spo_run(j->net, j->warmup);
	long long e0 = spo_events(j->net);
	pthread_barrier_wait(j->bar);
	spo_run(j->net, j->steps);
	j->events = spo_events(j->net) - e0;
	pthread_barrier_wait(j->bar);
	return NULL;
}

int main(int argc, char** argv) {
	if (argc < 6) {
		fprintf(stderr, "usage: oracle_bench N P STEPS SEED0 THREADS [WARMUP]\n");
		return 2;
	}
	long long N = atoll(argv[1]);
	double p    = atof(argv[2]);
	long long steps = atoll(argv[3]);
	unsigned seed0  = (unsigned)atoll(argv[4]);
	int T           = atoi(argv[5]);
	long long warm  = argc > 6 ? atoll(argv[6]) : 0;
	if (T < 1) T = 1;
	pthread_barrier_t bar;
	pthread_barrier_init(&bar, NULL, (unsigned)T + 1);
	job* jobs      = (job*)calloc((size_t)T, sizeof(job));
	pthread_t* th  = (pthread_t*)calloc((size_t)T, sizeof(pthread_t));
	for (int i = 0; i < T; i++) {
		jobs[i] = (job){N, steps, warm, p, seed0 + (unsigned)i, 0, 0, 0, NULL, &bar};
		pthread_create(&th[i], NULL, worker, &jobs[i]);
	}
	pthread_barrier_wait(&bar);
	double t0 = now();
	pthread_barrier_wait(&bar);
	double t1 = now();
	long long ev = 0;
	double build = 0;
	for (int i = 0; i < T; i++) {
		pthread_join(th[i], NULL);
		ev += jobs[i].events;
		build = build > jobs[i].build_s ? build : jobs[i].build_s;
		spo_net_destroy(jobs[i].net);
	}
	double dt = t1 - t0;
	printf("{\"events\": %lld, \"step_seconds\": %.6f, \"build_seconds\": %.6f, \"threads\": %d, "
	       "\"steps\": %lld, \"N\": %lld, \"p\": %g, \"events_per_s\": %.6g, \"ms_per_step\": %.6f}\n",
	       ev, dt, build, T, steps, N, p, ev / dt, 1e3 * dt / (double)steps);
	free(jobs);
	free(th);
	return 0;
}
