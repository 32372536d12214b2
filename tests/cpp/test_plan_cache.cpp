// Host-only unit test of the autotuner's plan cache file
// (glscv_gb300/csrc/plan_cache.h): line format, parser, escapes, lookup of
// the last matching line, skipping of malformed lines, appends.
#include <cstdio>
#include <string>

#include "plan_cache.h"

namespace pc = glsfft::plan_cache;

static int failures = 0;
#define EXPECT(c)                                                   \
    do {                                                            \
        if (!(c)) {                                                 \
            std::printf("FAIL line %d: %s\n", __LINE__, #c);        \
            failures++;                                             \
        }                                                           \
    } while (0)

int main(int argc, char **argv) {
    const std::string path = argc > 1 ? argv[1] : "plan_cache_test.jsonl";
    std::remove(path.c_str());

    // format -> parse round trip, with escapes and numbers
    pc::Pairs kv = {{"device", pc::quote("NVIDIA \"GB300\" \\ x")},
                    {"sms", "152"},
                    {"ms", "0.8971"},
                    {"neg", "-3e-05"},
                    {"ok", "true"}};
    const std::string line = pc::format_line(kv);
    pc::Fields f;
    EXPECT(pc::parse_line(line, f));
    EXPECT(f["device"] == "NVIDIA \"GB300\" \\ x");
    EXPECT(f["sms"] == "152" && f["ms"] == "0.8971" && f["neg"] == "-3e-05" && f["ok"] == "true");
    EXPECT(pc::quote(std::string("a\nb")) == "\"a\\u000ab\"");
    EXPECT(pc::parse_line("{\"s\": \"a\\u000ab\\tc\"}", f) && f["s"] == "a\nb\tc");
    EXPECT(pc::parse_line("  {}  ", f) && f.empty());

    // malformed lines are rejected
    EXPECT(!pc::parse_line("", f));
    EXPECT(!pc::parse_line("{\"a\": 1", f));
    EXPECT(!pc::parse_line("{\"a\": [1, 2]}", f));
    EXPECT(!pc::parse_line("{\"a\": {\"b\": 1}}", f));
    EXPECT(!pc::parse_line("{\"a\" 1}", f));
    EXPECT(!pc::parse_line("{\"a\": 1} trailing", f));
    EXPECT(!pc::parse_line("{\"a\": \"\\u00e9\"}", f));  // only ASCII escapes are decoded

    // lookup on a missing file finds nothing
    pc::Fields hit;
    EXPECT(!pc::lookup(path.c_str(), {{"kind", "fft2d"}}, hit));
    EXPECT(!pc::lookup(nullptr, {}, hit));
    EXPECT(!pc::append(nullptr, kv));

    // appends; the last matching line wins; torn / foreign lines are skipped
    EXPECT(pc::append(path.c_str(), {{"kind", pc::quote("fft2d")}, {"rows", "1024"},
                                     {"cols", "1024"}, {"row_schedule", "1"}}));
    EXPECT(pc::append(path.c_str(), {{"kind", pc::quote("fft2d")}, {"rows", "512"},
                                     {"cols", "512"}, {"row_schedule", "3"}}));
    {
        std::FILE *fp = std::fopen(path.c_str(), "a");
        std::fputs("{\"kind\": \"fft2d\", \"rows\": 1024, \"cols\": 10\n", fp);  // torn
        std::fputs("not json at all\n", fp);
        std::fputs("\n", fp);
        std::fclose(fp);
    }
    EXPECT(pc::append(path.c_str(), {{"kind", pc::quote("fft2d")}, {"rows", "1024"},
                                     {"cols", "1024"}, {"row_schedule", "4"}}));
    const pc::Fields want = pc::as_fields({{"kind", pc::quote("fft2d")}, {"rows", "1024"},
                                           {"cols", "1024"}});
    EXPECT(want.at("kind") == "fft2d" && want.at("rows") == "1024");
    EXPECT(pc::lookup(path.c_str(), want, hit) && hit["row_schedule"] == "4");
    EXPECT(pc::lookup(path.c_str(), {{"rows", "512"}}, hit) && hit["row_schedule"] == "3");
    EXPECT(!pc::lookup(path.c_str(), {{"rows", "2048"}}, hit));
    EXPECT(!pc::lookup(path.c_str(), {{"kind", "batch"}}, hit));

    // a long line (a batch plan's histogram) survives the line reader
    std::string hist;
    for (int i = 0; i < 600; i++) hist += "1024x1024*" + std::to_string(i) + ";";
    EXPECT(pc::append(path.c_str(), {{"kind", pc::quote("batch")}, {"persistent", pc::quote(hist)},
                                     {"variant", "2"}}));
    EXPECT(pc::lookup(path.c_str(), {{"kind", "batch"}, {"persistent", hist}}, hit) &&
           hit["variant"] == "2");

    std::remove(path.c_str());
    if (failures) return 1;
    std::printf("ALL OK\n");
    return 0;
}
