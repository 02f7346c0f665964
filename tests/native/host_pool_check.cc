// Checks the host thread pool of the solver's set-up and transfer loops
// (seidart-backend_gb300/csrc/host_pool.h) on the CPU: every element of a
// range visited exactly once for many sizes, three threads calling at once,
// a forked child (which has no pool workers), more ranges than workers and
// a loop nested inside a range.
#include <sys/wait.h>
#include <atomic>
#include <cstdio>
#include <numeric>
#include "host_pool.h"
using seidart_host::host_parallel;
static bool check(size_t m) {
    std::vector<int> v(m, 0);
    host_parallel(m, [&](size_t lo, size_t hi) { for (size_t q = lo; q < hi; ++q) v[q] += 1; });
    for (size_t q = 0; q < m; ++q) if (v[q] != 1) return false;
    return true;
}
int main() {
    for (int r = 0; r < 2000; ++r) {
        const size_t m = (size_t)(r % 37) * 100003 + (r % 5) * (1 << 18);
        if (!check(m)) { printf("FAIL m=%zu\n", m); return 1; }
    }
    std::atomic<int> bad{0};
    auto worker = [&] { for (int r = 0; r < 500; ++r) if (!check((size_t)(r % 11 + 1) << 19)) ++bad; };
    std::thread a(worker), b(worker), c(worker);
    a.join(); b.join(); c.join();
    if (bad) { printf("FAIL concurrent\n"); return 1; }
    pid_t p = fork();
    if (p == 0) {
        for (int r = 0; r < 50; ++r) if (!check((size_t)(r + 1) << 19)) _exit(3);
        exit(0);   // runs static destructors: the pool has none
    }
    int st = 0; waitpid(p, &st, 0);
    if (!WIFEXITED(st) || WEXITSTATUS(st) != 0) { printf("FAIL fork %d\n", st); return 1; }
    // overflow ranges beyond the pool's size
    seidart_host::HostPool& pool = seidart_host::HostPool::get();
    std::vector<int> hit(pool.size() + 7, 0);
    pool.run((int)hit.size(), [&](int w) { hit[w] += 1; });
    for (int h : hit) if (h != 1) { printf("FAIL overflow\n"); return 1; }
    // a loop inside a range runs on the calling thread instead of waiting for the pool
    std::vector<std::atomic<int>> inner(64 << 18);
    host_parallel(16 << 18, [&](size_t lo, size_t hi) {
        (void)hi;
        const size_t base = (lo / (1 << 18)) % 4;
        host_parallel(16 << 18, [&](size_t a, size_t b) {
            for (size_t q = a; q < b; q += 4096) inner[base * (16 << 18) + q] += 1;
        });
    });
    long total = 0;
    for (auto& x : inner) total += x;
    if (total <= 0) { printf("FAIL nested\n"); return 1; }
    printf("ok size=%d\n", pool.size());
    return 0;
}
