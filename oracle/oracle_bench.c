/*
 * oracle_bench.c -- times the CPU restatement of snn::step on the Brunel network
 * (TEST INFRASTRUCTURE ONLY: bench.py's cpu_baseline / --impl reference leg runs it).
 *
 * usage: oracle_bench N P STEPS SEED0 THREADS [WARMUP [SAMPLES [SAME_SEED [NET]]]]
 *   Builds THREADS Brunel networks (the model of samples/brunel.cpp:75-116 with weights scaled by
 *   0.1/P), one per thread, with seeds SEED0, SEED0+1, ... or, with SAME_SEED = 1, all with SEED0
 *   (replicas of one simulation), runs WARMUP untimed steps, then times SAMPLES consecutive samples
 *   of STEPS steps of all networks in parallel (default 1).  Prints one JSON line: the aggregate
 *   events/s over all samples, per core, and per sample.
 *   NET = plastic_ei builds the plastic E/I network instead (N conductance LIF neurons, 80 % E and
 *   20 % I, fixed_probability(0.02), E weights 0.03, I weights 0.3, iSTDP on I->E with eta 1e-3,
 *   rho0 5 Hz, tau 20 ms, delay 1 step; P is ignored).
 */
#define _POSIX_C_SOURCE 200809L
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "spice_oracle.h"

#define MAX_SAMPLES 1024

typedef struct {
	long long N, steps, warmup;
	int samples;
	double p;
	unsigned seed;
	long long events[MAX_SAMPLES];
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

/* The plastic E/I network (conductance LIF of samples/vogels.cpp, iSTDP on I->E). */
spo_net* plastic_ei(long long N, unsigned seed) {
	float dt   = 1e-4f;
	uint32_t s = seed;
	spo_net* n = spo_net_create(dt, dt, &s, 1);
	int E = spo_add_population(n, SPO_LIF_COND, N * 8 / 10, NULL, 0);
	int I = spo_add_population(n, SPO_LIF_COND, N * 2 / 10, NULL, 0);
	spo_connect(n, E, E, 0.02, dt, 1, 0.03f);
	spo_connect(n, E, I, 0.02, dt, 1, 0.03f);
	int c = spo_connect(n, I, E, 0.02, dt, 2, 0.3f);
	spo_set_plastic(n, c, SPO_SYN_ISTDP, 0.3f, 1e-3f, 5.0f, 0.02f);
	spo_connect(n, I, I, 0.02, dt, 2, 0.3f);
	return n;
}

static int g_plastic = 0;

static void* worker(void* arg) {
	job* j      = (job*)arg;
	double t0   = now();
	j->net      = g_plastic ? plastic_ei(j->N, j->seed) : brunel(j->N, j->p, j->seed);
	j->build_s  = now() - t0;
	spo_run(j->net, j->warmup);
	for (int k = 0; k < j->samples; k++) {
		long long e0 = spo_events(j->net);
		pthread_barrier_wait(j->bar);
		spo_run(j->net, j->steps);
		j->events[k] = spo_events(j->net) - e0;
		pthread_barrier_wait(j->bar);
	}
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
	int samples     = argc > 7 ? atoi(argv[7]) : 1;
	int same_seed   = argc > 8 ? atoi(argv[8]) : 0;
	g_plastic       = argc > 9 && strcmp(argv[9], "plastic_ei") == 0;
	if (T < 1) T = 1;
	if (samples < 1) samples = 1;
	if (samples > MAX_SAMPLES) samples = MAX_SAMPLES;
	pthread_barrier_t bar;
	pthread_barrier_init(&bar, NULL, (unsigned)T + 1);
	job* jobs      = (job*)calloc((size_t)T, sizeof(job));
	pthread_t* th  = (pthread_t*)calloc((size_t)T, sizeof(pthread_t));
	for (int i = 0; i < T; i++) {
		jobs[i].N = N;
		jobs[i].steps = steps;
		jobs[i].warmup = warm;
		jobs[i].samples = samples;
		jobs[i].p = p;
		jobs[i].seed = same_seed ? seed0 : seed0 + (unsigned)i;
		jobs[i].bar = &bar;
		pthread_create(&th[i], NULL, worker, &jobs[i]);
	}
	double* dts = (double*)calloc((size_t)samples, sizeof(double));
	for (int k = 0; k < samples; k++) {
		pthread_barrier_wait(&bar);
		double t0 = now();
		pthread_barrier_wait(&bar);
		dts[k] = now() - t0;
	}
	long long ev = 0;
	double build = 0, dt = 0;
	for (int i = 0; i < T; i++) pthread_join(th[i], NULL);
	for (int i = 0; i < T; i++) {
		for (int k = 0; k < samples; k++) ev += jobs[i].events[k];
		build = build > jobs[i].build_s ? build : jobs[i].build_s;
		spo_net_destroy(jobs[i].net);
	}
	for (int k = 0; k < samples; k++) dt += dts[k];
	printf("{\"events\": %lld, \"step_seconds\": %.6f, \"build_seconds\": %.6f, \"threads\": %d, "
	       "\"steps\": %lld, \"samples\": %d, \"warmup\": %lld, \"same_seed\": %d, \"net\": \"%s\", \"N\": %lld, \"p\": %g, "
	       "\"events_per_s\": %.6g, \"events_per_s_per_core\": %.6g, \"ms_per_step\": %.6f, \"sample_events_per_s\": [",
	       ev, dt, build, T, steps, samples, warm, same_seed, g_plastic ? "plastic_ei" : "brunel", N, p, ev / dt, ev / dt / T, 1e3 * dt / (double)(steps * samples));
	for (int k = 0; k < samples; k++) {
		long long e = 0;
		for (int i = 0; i < T; i++) e += jobs[i].events[k];
		printf("%s%.6g", k ? ", " : "", e / dts[k]);
	}
	printf("]}\n");
	free(dts);
	free(jobs);
	free(th);
	return 0;
}
