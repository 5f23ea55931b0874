// gala_preprocess - text edge list -> .bin CSR.
// Drop-in for the reference `preprocess` (src/preprocess.cpp:7-47):
//     gala_preprocess -f <edges.txt> [-w] [-o <output_dir>]
// writes <edges.txt>.bin or <output_dir>/<name>.bin.  Parsing and row
// deduplication run on all cores (-j <threads> to limit them); weighted input
// keeps its summed weights (the reference writes only the first one,
// graph.cpp:132-143).
#include <stdio.h>
#include <stdlib.h>
#include <unistd.h>

#include <string>

#include "../../include/gala.h"

int main(int argc, char **argv)
{
    std::string input, out_dir;
    int weighted = 0, threads = 0, opt;
    while ((opt = getopt(argc, argv, "f:wo:j:")) != -1) {
        switch (opt) {
        case 'f': input = optarg; break;
        case 'w': weighted = 1; break;
        case 'o': out_dir = optarg; break;
        case 'j': threads = atoi(optarg); break;
        default:
            fprintf(stderr, "Usage: %s -f <filename> [-w -o <output_dirname>]\n", argv[0]);
            return 1;
        }
    }
    if (input.empty()) {
        printf("Input file not specified. Usage: %s -f <filename> [-w -o <output_dirname>]\n", argv[0]);
        return 1;
    }
    std::string output;
    if (!out_dir.empty()) {
        size_t p = input.find_last_of('/');
        output = out_dir + "/" + (p == std::string::npos ? input : input.substr(p + 1)) + ".bin";
    } else {
        output = input + ".bin";
    }
    printf("%s\n", output.c_str());
    gala_graph *g = nullptr;
    if (gala_graph_from_text(input.c_str(), weighted, threads, &g) != GALA_OK) {
        fprintf(stderr, "%s\n", gala_last_error());
        return 2;
    }
    int32_t n = 0;
    int64_t E = 0;
    gala_graph_info(g, &n, &E, nullptr);
    printf("vertex number:%d edge number:%lld\n", n, (long long)(E / 2));
    if (gala_graph_store_bin(g, output.c_str()) != GALA_OK) {
        fprintf(stderr, "%s\n", gala_last_error());
        gala_graph_destroy(g);
        return 3;
    }
    gala_graph_destroy(g);
    printf("store successfully. \n");
    return 0;
}
