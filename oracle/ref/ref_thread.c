/* POSIX-threads stand-in for the reference's Win32 thread pool (tay/thread.c).
 *
 * Test infrastructure only: the oracle recipe links this file in place of tay/thread.c,
 * which includes <windows.h> (tay/thread.c:8) and cannot build on Linux.  It implements
 * the interface declared by the reference's tay/thread.h with the same observable
 * behaviour:
 *   - tay_threads_start(n, storage): n workers (0 = all online cores, capped at
 *     TAY_MAX_THREADS), each with `storage` bytes of zeroed per-thread storage
 *     (tay/thread.c:70-76, 51-68);
 *   - tay_thread_set_task / tay_runner_run: every worker runs its task once and the
 *     caller blocks until all have finished (tay/thread.c:78-89);
 *   - tay_threads_range: the static split of [0, count) used by every pass
 *     (tay/thread.c:244-250): equal shares, the last thread takes the remainder.
 * Telemetry is compiled out in the reference build (TAY_TELEMETRY 0, tay/config.h:13),
 * so the telemetry entry points are no-ops here. */
#include "thread.h"
#include "state.h"
#include "tay.h"

#include <pthread.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <unistd.h>

TayRunner runner;

typedef struct {
    pthread_t handle;
    int index;
    unsigned long long start_generation; /* generation current when the worker was created */
} RefWorker;

static RefWorker workers[TAY_MAX_THREADS];
static pthread_mutex_t pool_lock = PTHREAD_MUTEX_INITIALIZER;
static pthread_cond_t pool_go = PTHREAD_COND_INITIALIZER;
static pthread_cond_t pool_done = PTHREAD_COND_INITIALIZER;
static unsigned long long pool_generation = 0;
static int pool_remaining = 0;

static void *worker_main(void *arg) {
    RefWorker *w = (RefWorker *)arg;
    TayThread *t = runner.threads + w->index;
    unsigned long long seen = w->start_generation;
    for (;;) {
        pthread_mutex_lock(&pool_lock);
        while (pool_generation == seen)
            pthread_cond_wait(&pool_go, &pool_lock);
        seen = pool_generation;
        int keep_running = t->run;
        pthread_mutex_unlock(&pool_lock);

        if (keep_running && t->task_func)
            t->task_func(t->task, &t->context);

        pthread_mutex_lock(&pool_lock);
        if (--pool_remaining == 0)
            pthread_cond_signal(&pool_done);
        pthread_mutex_unlock(&pool_lock);

        if (!keep_running)
            return 0;
    }
}

static void run_generation(void) {
    pthread_mutex_lock(&pool_lock);
    pool_remaining = runner.count;
    ++pool_generation;
    pthread_cond_broadcast(&pool_go);
    while (pool_remaining > 0)
        pthread_cond_wait(&pool_done, &pool_lock);
    pthread_mutex_unlock(&pool_lock);
}

void tay_threads_start(unsigned threads_count, unsigned thread_storage_size) {
    if (runner.state != TAY_RUNNER_IDLE)
        return;
    if (threads_count == 0) {
        long online = sysconf(_SC_NPROCESSORS_ONLN);
        threads_count = online > 0 ? (unsigned)online : 1u;
    }
    if (threads_count > TAY_MAX_THREADS)
        threads_count = TAY_MAX_THREADS;
    runner.thread_storage_size = thread_storage_size;
    runner.count = (int)threads_count;
    for (unsigned i = 0; i < threads_count; ++i) {
        TayThread *t = runner.threads + i;
        t->run = 1;
        t->task = 0;
        t->task_func = 0;
        t->context.storage = calloc(1, thread_storage_size ? thread_storage_size : 1);
        t->context.storage_size = thread_storage_size;
        workers[i].index = (int)i;
        workers[i].start_generation = pool_generation;
        pthread_create(&workers[i].handle, 0, worker_main, workers + i);
    }
    runner.state = TAY_RUNNER_WAITING;
}

void tay_threads_stop(void) {
    if (runner.state == TAY_RUNNER_IDLE)
        return;
    for (int i = 0; i < runner.count; ++i)
        runner.threads[i].run = 0;
    run_generation();
    for (int i = 0; i < runner.count; ++i) {
        pthread_join(workers[i].handle, 0);
        free(runner.threads[i].context.storage);
        runner.threads[i].context.storage = 0;
    }
    runner.count = 0;
    runner.state = TAY_RUNNER_IDLE;
}

unsigned tay_get_number_of_threads(void) {
    return (unsigned)runner.count;
}

void tay_thread_set_task(int index, void (*task_func)(TayThreadTask *, TayThreadContext *), TayThreadTask *task, void *context) {
    TayThread *t = runner.threads + index;
    t->task = task;
    t->task_func = task_func;
    t->context.context = context;
}

void tay_runner_run(void) {
    run_generation();
}

void tay_runner_run_no_threads(void) {
    for (int i = 0; i < runner.count; ++i) {
        TayThread *t = runner.threads + i;
        t->task_func(t->task, &t->context);
    }
}

void tay_threads_update_telemetry(void) {}
void tay_threads_report_telemetry(unsigned steps_between_reports, void *file) {
    (void)steps_between_reports;
    (void)file;
}
void tay_threads_get_telemetry_results(TayTelemetryResults *results) {
    (void)results;
}

TayRange tay_threads_range(unsigned count, unsigned thread_i) {
    TayRange r;
    unsigned share = count / (unsigned)runner.count;
    r.beg = share * thread_i;
    r.end = (thread_i + 1u < (unsigned)runner.count) ? r.beg + share : count;
    return r;
}

void tay_log(void *file, char *fmt, ...) {
    (void)file;
    (void)fmt;
}
