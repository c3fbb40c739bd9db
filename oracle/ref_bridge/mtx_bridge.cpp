// C-linkage wrapper around the reference's Matrix Market reader, readMtx<float>
// (gcn/util/util.hpp:286-333, with makeSymmetric :218-284 and the NIST parsers of
// gcn/util/mmio.hpp). Returns the three vectors readMtx leaves (row, column, value), in the
// order it leaves them, in malloc'd arrays the caller frees with ref_mtx_free. The reference
// headers are compiled from where they lie; mmio.hpp defines its functions, so this is the
// only translation unit that includes it. Test infrastructure only.
#include <cstdlib>
#include <cstring>
#include <vector>

#include "util.hpp"

extern "C" {
int ref_read_mtx(const char *path, int *nrows, int *ncols, int *nvals, int **rows, int **cols,
                 float **vals) {
    std::vector<int> r, c;
    std::vector<float> v;
    int m = 0, n = 0, nz = 0;
    readMtx<float>(path, r, c, v, m, n, nz);
    const size_t len = r.size();
    *nrows = m;
    *ncols = n;
    *nvals = static_cast<int>(len);
    *rows = static_cast<int *>(malloc(sizeof(int) * (len ? len : 1)));
    *cols = static_cast<int *>(malloc(sizeof(int) * (len ? len : 1)));
    *vals = static_cast<float *>(malloc(sizeof(float) * (len ? len : 1)));
    if (len) {
        memcpy(*rows, r.data(), sizeof(int) * len);
        memcpy(*cols, c.data(), sizeof(int) * len);
        memcpy(*vals, v.data(), sizeof(float) * std::min(len, v.size()));
    }
    return static_cast<int>(v.size());
}
void ref_mtx_free(void *p) { free(p); }
}
