// Known-answer vectors of the libstdc++ random facilities the PT-ICM
// reference draws from (std::mt19937_64, uniform_real_distribution<double>,
// bernoulli_distribution, std::shuffle, std::sample).  Built and run by
// make_golden.py with the system g++; its output is tests/golden/rng_kat.json.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <random>
#include <vector>

int main() {
    std::printf("{\n");
    {
        std::mt19937_64 g;  // default seed 5489
        std::uint64_t v = 0;
        for (int i = 0; i < 10000; i++) v = g();
        std::printf("  \"mt64_default_10000th\": \"%llu\",\n", (unsigned long long)v);
    }
    {
        std::mt19937_64 g(12345);
        std::printf("  \"mt64_seed12345_first8\": [");
        for (int i = 0; i < 8; i++) std::printf("%s\"%llu\"", i ? ", " : "", (unsigned long long)g());
        std::printf("],\n");
    }
    {
        std::mt19937_64 g(7);
        std::uniform_real_distribution<double> u(0, 1);
        std::printf("  \"canonical_seed7_first16\": [");
        for (int i = 0; i < 16; i++) std::printf("%s%.17g", i ? ", " : "", u(g));
        std::printf("],\n");
    }
    {
        std::mt19937_64 g(99);
        std::bernoulli_distribution b(0.5);
        std::printf("  \"bernoulli_seed99_first64\": [");
        for (int i = 0; i < 64; i++) std::printf("%s%d", i ? ", " : "", (int)b(g));
        std::printf("],\n");
    }
    {
        std::mt19937_64 g(2024);
        std::printf("  \"shuffle_seed2024\": [");
        int first = 1;
        for (int n : {1, 2, 3, 7, 8, 31, 63, 64}) {
            std::vector<std::uint32_t> a(n);
            for (int i = 0; i < n; i++) a[i] = i;
            std::shuffle(a.begin(), a.end(), g);
            std::printf("%s[", first ? "" : ", ");
            first = 0;
            for (int i = 0; i < n; i++) std::printf("%s%u", i ? ", " : "", a[i]);
            std::printf("]");
        }
        std::printf("],\n");
    }
    {
        std::mt19937_64 g(31337);
        std::printf("  \"sample1_seed31337\": [");
        int first = 1;
        for (int n : {1, 2, 3, 5, 10, 100, 401, 1000, 2, 1, 77}) {
            std::vector<std::int64_t> pop(n);
            for (int i = 0; i < n; i++) pop[i] = i;
            std::vector<std::int64_t> out(1);
            std::sample(pop.begin(), pop.end(), out.begin(), 1, g);
            std::printf("%s[%d, %lld]", first ? "" : ", ", n, (long long)out[0]);
            first = 0;
        }
        std::printf("]\n");
    }
    std::printf("}\n");
    return 0;
}
