// gala_main - command line front end of the GB300 Louvain engine.
// Drop-in for the reference CLI (src/gala_main.cu:8-57):
//     gala_main -f <graph.bin> [-w]
// prints the reference's per-round / per-iteration lines (README.md:59-89).
// Extra options: -o <file> writes the final community of every vertex (one
// int32 per vertex, binary), -t <threshold> (default 1e-6), -l <max rounds>,
// -d <device>, -s <dir> writes every round's contracted graph and labels
// (checkpoints to resume from), -r turns on the Leiden-style refinement.
#include <stdio.h>
#include <stdlib.h>
#include <sys/time.h>
#include <unistd.h>

#include <vector>

#include "../../include/gala.h"

static double now_ms()
{
    struct timeval t;
    gettimeofday(&t, nullptr);
    return (double)t.tv_sec * 1000 + (double)t.tv_usec / 1000;
}

int main(int argc, char **argv)
{
    const char *file = nullptr, *out = nullptr;
    int weighted = 0, device = 0, opt;
    gala_options o;
    gala_default_options(&o);
    while ((opt = getopt(argc, argv, "f:wo:t:l:d:s:r")) != -1) {
        switch (opt) {
        case 'f': file = optarg; break;
        case 'w': weighted = 1; break;
        case 'o': out = optarg; break;
        case 't': o.min_modularity = atof(optarg); break;
        case 'l': o.max_levels = atoi(optarg); break;
        case 'd': device = atoi(optarg); break;
        case 's': o.level_dir = optarg; break;
        case 'r': o.refine = 1; break;
        default:
            fprintf(stderr,
                    "Usage: %s -f <graph.bin> [-w] [-o labels.bin] [-t threshold] [-l rounds] [-d device] "
                    "[-s level_dir] [-r]\n",
                    argv[0]);
            return 1;
        }
    }
    if (!file) {
        fprintf(stderr, "Usage: %s -f <graph.bin> [-w]\n", argv[0]);
        return 1;
    }
    double start = now_ms();
    gala_graph *g = nullptr;
    gala_status s = gala_graph_load_bin(file, weighted, &g);
    if (s != GALA_OK) {
        fprintf(stderr, "load failed: %s\n", gala_last_error());
        return 2;
    }
    int32_t n = 0;
    int64_t E = 0;
    gala_graph_info(g, &n, &E, nullptr);
    printf("vertex number:%d edge number:%lld\n", n, (long long)(E / 2));
    printf("load success\n");
    gala_context *ctx = nullptr;
    if ((s = gala_context_create(device, n, E, &ctx)) != GALA_OK) {
        fprintf(stderr, "device setup failed: %s\n", gala_last_error());
        gala_graph_destroy(g);
        return 3;
    }
    std::vector<int32_t> comm(n);
    gala_result r{};
    o.verbose = 1;
    s = gala_louvain(ctx, g, &o, comm.data(), &r);
    if (s != GALA_OK) {
        fprintf(stderr, "louvain failed: %s\n", gala_last_error());
        gala_context_destroy(ctx);
        gala_graph_destroy(g);
        return 4;
    }
    if (out) {
        FILE *f = fopen(out, "wb");
        if (!f || fwrite(comm.data(), sizeof(int32_t), comm.size(), f) != comm.size()) {
            fprintf(stderr, "cannot write %s\n", out);
            if (f) fclose(f);
            return 5;
        }
        fclose(f);
    }
    gala_context_destroy(ctx);
    gala_graph_destroy(g);
    double end = now_ms();
    printf("elapsed time = %fms\n", end - start);
    return 0;
}
