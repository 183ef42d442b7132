// args.h -- the command-line convention of the PaRGO application mains:
// either flags (-elev FILE -nbr FILE -out FILE [-mtd M] [-dirtype T]) or the
// positional form (elev nbr out [extra]).
#ifndef PARGO_APPS_ARGS_H
#define PARGO_APPS_ARGS_H
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

struct AppArgs {
    const char* elev = nullptr;
    const char* nbr = nullptr;
    const char* out = nullptr;
    const char* extra = nullptr;  // -mtd / -dirtype / 4th positional
};

// `out_flag` is the flag naming the output ("-slp" for slope, "-out" otherwise);
// `extra_flag` the optional fourth argument's flag (or nullptr).
inline bool parse_app_args(int argc, char** argv, const char* out_flag, const char* extra_flag, AppArgs* a,
                           std::string* err) {
    bool flags = false, positional = false;
    for (int i = 1; i < argc; i++) {
        const char* s = argv[i];
        auto take = [&](const char** dst) {
            if (i + 1 >= argc) {
                *err = std::string("no argument after ") + s;
                return false;
            }
            *dst = argv[++i];
            flags = true;
            return true;
        };
        if (!strcmp(s, "-elev")) { if (!take(&a->elev)) return false; }
        else if (!strcmp(s, "-nbr")) { if (!take(&a->nbr)) return false; }
        else if (!strcmp(s, out_flag) || !strcmp(s, "-out")) { if (!take(&a->out)) return false; }
        else if (extra_flag && !strcmp(s, extra_flag)) { if (!take(&a->extra)) return false; }
        else {
            if (flags) {
                *err = "do not mix the flag and positional forms";
                return false;
            }
            positional = true;
            a->elev = argv[1];
            a->nbr = argc > 2 ? argv[2] : nullptr;
            a->out = argc > 3 ? argv[3] : nullptr;
            a->extra = argc > 4 ? argv[4] : nullptr;
            break;
        }
    }
    (void)positional;
    if (!a->elev || !a->nbr || !a->out) {
        *err = "input, neighbourhood and output files are required";
        return false;
    }
    return true;
}
#endif
