/* A plain C99 client of the library's C ABI: the headers compile as C, every entry point links, and the host-side
 * functions run without a GPU.  It parses a solidDict, turns its solids into states and prints the cloud.out records
 * and the size of the restart dictionary; the CUDA entry points are only linked (their addresses are taken).
 *
 *   client SOLIDDICT */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "sdfibm_cuda.h"
#include "sdfibm_host.h"
#include "sdfibm_mlp.h"

static char* slurp(const char* path) {
    FILE* f = fopen(path, "rb");
    if (!f) return NULL;
    fseek(f, 0, SEEK_END);
    long n = ftell(f);
    fseek(f, 0, SEEK_SET);
    char* t = (char*)malloc((size_t)n + 1);
    if (t && fread(t, 1, (size_t)n, f) != (size_t)n) { free(t); t = NULL; }
    if (t) t[n] = 0;
    fclose(f);
    return t;
}

int main(int argc, char** argv) {
    /* the CUDA entry points link (not called: no GPU is needed here) */
    typedef void (*entry_fn)(void);
    entry_fn entry[] = {(entry_fn)sdfibm_cuda_create, (entry_fn)sdfibm_cuda_interact,
                        (entry_fn)sdfibm_cuda_interact_host, (entry_fn)sdfibm_cuda_interact_host64,
                        (entry_fn)sdfibm_cuda_create_polymesh, (entry_fn)sdfibm_cuda_tuning,
                        (entry_fn)sdfibm_cuda_evolve,
                        (entry_fn)sdfibm_cuda_fix_internal, (entry_fn)sdfibm_cuda_get_solids,
                        (entry_fn)sdfibm_cuda_set_solids, (entry_fn)sdfibm_cuda_touched, (entry_fn)sdfibm_cuda_stats,
                        (entry_fn)sdfibm_cuda_destroy, (entry_fn)sdfibm_cuda_set_fraction_model,
                        (entry_fn)sdfibm_mlp_train};
    size_t linked = 0, i;
    for (i = 0; i < sizeof(entry) / sizeof(entry[0]); ++i) linked += entry[i] != NULL;

    if (argc < 2) return 5;
    char* dict = slurp(argv[1]);
    if (!dict) return 6;
    sdfibm_options opt;
    sdfibm_solid_desc solids[4];
    int32_t n = 0, twod = -1;
    char msg[256];
    if (sdfibm_host_parse_soliddict(dict, 1000.0, solids, 4, &n, &opt, &twod, msg, (int32_t)sizeof(msg)) !=
        SDFIBM_OK) {
        fprintf(stderr, "parse: %s\n", msg);
        return 1;
    }
    sdfibm_solid_state st[4];
    memset(st, 0, sizeof(st));
    for (i = 0; i < (size_t)n; ++i) {
        memcpy(st[i].pos, solids[i].pos, sizeof(st[i].pos));
        memcpy(st[i].quat, solids[i].quat, sizeof(st[i].quat));
        memcpy(st[i].vel, solids[i].vel, sizeof(st[i].vel));
        memcpy(st[i].omega, solids[i].omega, sizeof(st[i].omega));
    }
    int64_t len = 0;
    if (sdfibm_host_format_state(0.5, twod, st, n, NULL, 0, &len) != SDFIBM_OK) return 2;
    char* text = (char*)malloc((size_t)len + 1);
    if (!text || sdfibm_host_format_state(0.5, twod, st, n, text, len + 1, &len) != SDFIBM_OK) return 3;
    int64_t rlen = 0;
    if (sdfibm_host_write_restart(dict, st, n, twod, 6, "stamp", NULL, 0, &rlen, msg, (int32_t)sizeof(msg)) !=
        SDFIBM_OK) {
        fprintf(stderr, "restart: %s\n", msg);
        return 4;
    }
    printf("linked %zu\nsolids %d twod %d rho_f %g\nrestart %lld\n%s", linked, (int)n, (int)twod, opt.rho_f,
           (long long)rlen, text);
    free(text);
    free(dict);
    return 0;
}
