// Host-only checks of the autotuner's cache file (pargo_gb300/csrc/tune_cache.h):
// write/read round trips, malformed and foreign content, the path rules and
// the write through a temporary file, also from two threads at once.
// Usage: tune_cache_check <scratch dir>.
// Prints one line per failed check and exits non-zero if any failed.
#include "tune_cache.h"

#include <dirent.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

using pargo::TuneEntry;

static int g_failed = 0;

#define CHECK(cond)                                                      \
    do {                                                                 \
        if (!(cond)) {                                                   \
            std::printf("FAILED line %d: %s\n", __LINE__, #cond);        \
            g_failed++;                                                  \
        }                                                                \
    } while (0)

static void put(const std::string& path, const std::string& text) {
    FILE* f = std::fopen(path.c_str(), "wb");
    std::fwrite(text.data(), 1, text.size(), f);
    std::fclose(f);
}

static TuneEntry entry(const char* op, const char* dev, int sc, const char* var, double ms) {
    TuneEntry e;
    e.op = op;
    e.device = dev;
    e.size_class = sc;
    e.variant = var;
    e.ms = ms;
    return e;
}

static int files_in(const std::string& dir) {
    int n = 0;
    if (DIR* d = opendir(dir.c_str())) {
        while (dirent* e = readdir(d))
            if (std::strcmp(e->d_name, ".") && std::strcmp(e->d_name, "..")) n++;
        closedir(d);
    }
    return n;
}

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    const std::string dir = argv[1];

    // round trip through a directory that does not exist yet; quotes and
    // backslashes survive, a control character becomes a space
    const std::string path = dir + "/a/b/tune.json";
    std::vector<TuneEntry> v = {entry("slope_d8", "sm_103 152 NVIDIA \"GB300\" \\x", 30, "strip-s6x8-b5", 2.031),
                                entry("slope_d8", "dev\tname", 20, "tiled-16x64", 0.125),
                                entry("other_op", "d", 0, "v", 1e-3)};
    CHECK(pargo::write_tune_cache(path, v));
    CHECK(files_in(dir + "/a/b") == 1);  // the temporary file was renamed away
    std::vector<TuneEntry> r = pargo::read_tune_cache(path);
    CHECK(r.size() == 3);
    if (r.size() == 3) {
        CHECK(r[0].op == "slope_d8" && r[0].device == v[0].device && r[0].size_class == 30 &&
              r[0].variant == "strip-s6x8-b5" && r[0].ms == 2.031);
        CHECK(r[1].device == "dev name" && r[1].size_class == 20 && r[1].ms == 0.125);
        CHECK(r[2].op == "other_op" && r[2].size_class == 0 && r[2].ms == 1e-3);
    }
    // rewriting replaces the file
    CHECK(pargo::write_tune_cache(path, std::vector<TuneEntry>(1, v[2])));
    CHECK(pargo::read_tune_cache(path).size() == 1);

    // no file, an empty path, an empty object, empty entries
    CHECK(pargo::read_tune_cache(dir + "/none.json").empty());
    CHECK(pargo::read_tune_cache("").empty());
    CHECK(!pargo::write_tune_cache("", v));
    const std::string p2 = dir + "/t.json";
    put(p2, "{}");
    CHECK(pargo::read_tune_cache(p2).empty());
    put(p2, "{\"version\": 1, \"entries\": []}");
    CHECK(pargo::read_tune_cache(p2).empty());

    // foreign keys and values of every kind are skipped, before and inside entries
    put(p2,
        "{\"tool\": {\"name\": \"x\", \"list\": [1, -2.5e3, true, false, null, [], {}, [\"s\\\"q\", {\"k\": [null]}]]},"
        " \"entries\": [{\"op\": \"a\", \"extra\": {\"deep\": [1, 2]}, \"device\": \"d\", \"size_class\": 12,"
        " \"variant\": \"v\\u00e9w\", \"ms\": 0.5, \"note\": null}], \"trailer\": \"t\"}");
    r = pargo::read_tune_cache(p2);
    CHECK(r.size() == 1);
    if (r.size() == 1) CHECK(r[0].op == "a" && r[0].size_class == 12 && r[0].variant == "v?w" && r[0].ms == 0.5);

    // entries without an operation or a variant, or with a size class out of
    // [0, 64), are dropped; the others are kept
    put(p2,
        "{\"entries\": [{\"device\": \"d\", \"size_class\": 3, \"variant\": \"v\"},"
        " {\"op\": \"a\", \"size_class\": 64, \"variant\": \"v\"}, {\"op\": \"a\", \"size_class\": -1, \"variant\": \"v\"},"
        " {\"op\": \"a\", \"size_class\": 5}, {\"op\": \"b\", \"size_class\": 7, \"variant\": \"w\"}]}");
    r = pargo::read_tune_cache(p2);
    CHECK(r.size() == 1 && r[0].op == "b" && r[0].size_class == 7);

    // malformed text ends the read; the entries read before it are kept
    const char* bad[] = {
        "{\"entries\": [{\"op\": \"a\", \"size_class\": 1, \"variant\": \"v\"}, {\"op\": \"b\", \"size_class\": ",
        "{\"entries\": [{\"op\": \"a\", \"size_class\": 1, \"variant\": \"v\"}, {\"op\" \"b\"}]}",
        "{\"entries\": [{\"op\": \"a\", \"size_class\": 1, \"variant\": \"v\"}, {\"op\": \"b\", \"size_class\": x}]}",
        "{\"entries\": [{\"op\": \"a\", \"size_class\": 1, \"variant\": \"v\"}, {\"op\": \"unterminated}]}",
    };
    for (const char* text : bad) {
        put(p2, text);
        r = pargo::read_tune_cache(p2);
        CHECK(r.size() == 1 && r[0].op == "a");
    }
    // not JSON at all, and nesting deeper than the reader follows
    put(p2, "not json");
    CHECK(pargo::read_tune_cache(p2).empty());
    put(p2, "{\"pad\": " + std::string(100000, '[') + "], \"entries\": [{\"op\": \"a\", \"size_class\": 1, \"variant\": \"v\"}]}");
    CHECK(pargo::read_tune_cache(p2).empty());
    put(p2, "{\"pad\": " + std::string(40, '[') + std::string(40, ']') +
                ", \"entries\": [{\"op\": \"a\", \"size_class\": 1, \"variant\": \"v\"}]}");
    CHECK(pargo::read_tune_cache(p2).size() == 1);

    // writers in two threads: every read sees one writer's whole file, and no
    // temporary file is left behind
    {
        const std::string p3 = dir + "/c/tune.json";
        const std::vector<TuneEntry> va(3, entry("a", "d", 1, "v", 1.0)), vb(5, entry("b", "d", 2, "w", 2.0));
        bool ok_a = true, ok_b = true;
        std::thread ta([&] { for (int k = 0; k < 200; k++) ok_a = pargo::write_tune_cache(p3, va) && ok_a; });
        std::thread tb([&] { for (int k = 0; k < 200; k++) ok_b = pargo::write_tune_cache(p3, vb) && ok_b; });
        int seen_bad = 0;
        for (int k = 0; k < 200; k++) {
            const std::vector<TuneEntry> got = pargo::read_tune_cache(p3);
            const bool whole = got.empty() || (got.size() == 3 && got[0].op == "a") || (got.size() == 5 && got[0].op == "b");
            seen_bad += whole ? 0 : 1;
        }
        ta.join();
        tb.join();
        CHECK(ok_a && ok_b);
        CHECK(seen_bad == 0);
        CHECK(files_in(dir + "/c") == 1);
    }

    // the cache path: PARGO_TUNE_CACHE (empty: no cache), else XDG_CACHE_HOME, else HOME
    setenv("PARGO_TUNE_CACHE", "/x/y.json", 1);
    CHECK(pargo::tune_cache_path() == "/x/y.json");
    setenv("PARGO_TUNE_CACHE", "", 1);
    CHECK(pargo::tune_cache_path().empty());
    unsetenv("PARGO_TUNE_CACHE");
    setenv("XDG_CACHE_HOME", "/xdg", 1);
    setenv("HOME", "/home/u", 1);
    CHECK(pargo::tune_cache_path() == "/xdg/pargo_gb300/tune.json");
    setenv("XDG_CACHE_HOME", "", 1);
    CHECK(pargo::tune_cache_path() == "/home/u/.cache/pargo_gb300/tune.json");
    unsetenv("XDG_CACHE_HOME");
    unsetenv("HOME");
    CHECK(pargo::tune_cache_path().empty());

    if (g_failed == 0) std::printf("ok\n");
    return g_failed ? 1 : 0;
}
