// Dump harness around the reference's own nstream and transpose drivers (test infrastructure only).
//
// The reference's drivers (Cxx11/nstream.cc, Cxx11/transpose.cc) print only their verdicts, and
// their arrays live inside main(). This harness includes one of them where it lies (PRK_SOURCE, with
// its main renamed), runs it unmodified with the caller's arguments, and keeps a copy of every array
// the driver allocates through prk::malloc (Cxx11/prk_util.h:159-196, posix_memalign) at the moment
// the driver frees it, i.e. after its last iteration. The copies go to a file in allocation order
// (nstream: A, B, C; transpose: A, B), each as an 8-byte little-endian byte count and the raw
// little-endian doubles. The link wraps posix_memalign and free (-Wl,--wrap) for the driver's calls
// only.
//
//   ref_nstream_dump   <iterations> <length> <dump.bin>
//   ref_transpose_dump <iterations> <order> [<tile>] <dump.bin>
#include <cstdio>
#include <cstdlib>
#include <utility>
#include <vector>

namespace {
std::vector<std::pair<void*, size_t>> g_blocks;  // the driver's arrays, in allocation order
std::vector<std::vector<char>> g_saved;          // their contents when freed
}  // namespace

extern "C" int __real_posix_memalign(void**, size_t, size_t);
extern "C" void __real_free(void*);

extern "C" int __wrap_posix_memalign(void** p, size_t alignment, size_t bytes)
{
    const int r = __real_posix_memalign(p, alignment, bytes);
    if (r == 0) {
        g_blocks.emplace_back(*p, bytes);
        g_saved.emplace_back();
    }
    return r;
}

extern "C" void __wrap_free(void* p)
{
    for (size_t k = 0; k < g_blocks.size(); ++k)
        if (p && g_blocks[k].first == p) {
            const char* c = static_cast<const char*>(p);
            g_saved[k].assign(c, c + g_blocks[k].second);
            g_blocks[k].first = nullptr;
        }
    __real_free(p);
}

#define main prk_reference_main
#include PRK_SOURCE
#undef main

int main(int argc, char* argv[])
{
    if (argc < 3) {
        std::fprintf(stderr, "usage: <the driver's arguments> <dump.bin>\n");
        return 2;
    }
    const char* path = argv[argc - 1];
    argv[argc - 1] = nullptr;
    const int rc = prk_reference_main(argc - 1, argv);
    FILE* f = std::fopen(path, "wb");
    if (!f) return 3;
    for (const auto& s : g_saved) {
        const unsigned long long bytes = s.size();
        std::fwrite(&bytes, sizeof bytes, 1, f);
        std::fwrite(s.data(), 1, s.size(), f);
    }
    std::fclose(f);
    return rc;
}
