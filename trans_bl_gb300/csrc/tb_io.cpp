// tb_io.cpp -- the reference's on-disk formats, so that a run on the GPU
// library and a run of the Fortran host can restart from each other's files
// and share post-processing.
//
//  data_XX.bin   checkpoint: escreve (escreve_par.f:6-31), read back at start
//                by init_fi (main_par.f:762-769):
//                  record 1: integer*4 t
//                  record 2: ux, uy, uz, wx, wy, wz   (complex*16 (nx, ny, kfour) each)
//  pert_XX_YY    snapshot for the temporal Fourier analysis: escreve2
//                (escreve_par.f:34-81): one record holding ux, with the base
//                flow uxb removed from the real part of mode 0 in form 0.
//
// Both are gfortran sequential unformatted files: every record is framed by
// 4-byte little-endian length markers, [n][payload][n].  A record longer than
// the largest subrecord (2^31 - 9 bytes) is written as a chain of subrecords;
// the leading marker of a subrecord is negated when another subrecord
// follows, the trailing marker is negated when one precedes it (the layout
// libgfortran documents for records over 2 GiB).
#include "tb_internal.h"
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

namespace {

long long g_subrec_max = 2147483639LL;   // gfortran's largest subrecord

bool put_i32(FILE* f, int v) {
    unsigned u;
    std::memcpy(&u, &v, 4);
    unsigned char b[4] = {(unsigned char)(u & 0xff), (unsigned char)((u >> 8) & 0xff), (unsigned char)((u >> 16) & 0xff),
                          (unsigned char)(u >> 24)};
    return fwrite(b, 1, 4, f) == 4;
}
bool get_i32(FILE* f, int* v) {
    unsigned char b[4];
    if (fread(b, 1, 4, f) != 4) return false;
    unsigned u = (unsigned)b[0] | ((unsigned)b[1] << 8) | ((unsigned)b[2] << 16) | ((unsigned)b[3] << 24);
    std::memcpy(v, &u, 4);
    return true;
}

// One logical record made of the concatenation of the given pieces.
struct Piece { const void* p; size_t n; };
int write_record(FILE* f, const std::vector<Piece>& pieces) {
    size_t total = 0;
    for (auto& q : pieces) total += q.n;
    size_t done = 0, pi = 0, po = 0;
    bool first = true;
    do {
        size_t len = (size_t)std::min<long long>((long long)(total - done), g_subrec_max);
        bool more = done + len < total;
        if (!put_i32(f, more ? -(int)len : (int)len)) return TB_ERR_ARG;
        size_t left = len;
        while (left > 0) {
            size_t take = std::min(left, pieces[pi].n - po);
            if (take && fwrite((const char*)pieces[pi].p + po, 1, take, f) != take) return TB_ERR_ARG;
            left -= take; po += take;
            if (po == pieces[pi].n) { pi++; po = 0; }
        }
        if (!put_i32(f, first ? (int)len : -(int)len)) return TB_ERR_ARG;
        done += len;
        first = false;
    } while (done < total);
    return TB_OK;
}

// Reads one logical record into dst (exactly n bytes expected).
int read_record(FILE* f, void* dst, size_t n, const char* what) {
    size_t got = 0;
    for (;;) {
        int head, tail;
        if (!get_i32(f, &head)) { tb_set_error("%s: truncated file (record marker)", what); return TB_ERR_ARG; }
        size_t len = (size_t)(head < 0 ? -(long long)head : head);
        if (got + len > n) { tb_set_error("%s: record holds more than the %zu bytes expected", what, n); return TB_ERR_ARG; }
        if (len && fread((char*)dst + got, 1, len, f) != len) { tb_set_error("%s: truncated record", what); return TB_ERR_ARG; }
        got += len;
        if (!get_i32(f, &tail)) { tb_set_error("%s: truncated file (record marker)", what); return TB_ERR_ARG; }
        if ((tail < 0 ? -(long long)tail : tail) != (long long)len) { tb_set_error("%s: record markers disagree", what); return TB_ERR_ARG; }
        if (head >= 0) break;
    }
    if (got != n) { tb_set_error("%s: record has %zu bytes, expected %zu (grid mismatch?)", what, got, n); return TB_ERR_ARG; }
    return TB_OK;
}

int download(tb_ctx* c, cplx* dev, std::vector<cplx>& h) {
    h.resize(tb_n3(c));
    TB_CUDA(cudaMemcpyAsync(h.data(), dev, h.size() * sizeof(cplx), cudaMemcpyDeviceToHost, c->stream));
    TB_CUDA(cudaStreamSynchronize(c->stream));
    return TB_OK;
}

}  // namespace

extern "C" {

int tb_io_set_subrecord_limit(long long bytes) {
    if (bytes < 8 || bytes > 2147483639LL) { tb_set_error("subrecord limit must be in [8, 2147483639]"); return TB_ERR_ARG; }
    g_subrec_max = bytes;
    return TB_OK;
}

// escreve (escreve_par.f:6-30): record 1 the step, record 2 ux uy uz wx wy
// wz, and th after them in the thermal form.
int tb_write_checkpoint(tb_ctx* c, const char* path, int t) {
    if (!c || !path) { tb_set_error("null argument"); return TB_ERR_ARG; }
    const int nf = c->cfg.my_form == 2 ? 7 : 6;
    std::vector<cplx> h[7];
    cplx* dev[7] = {c->ux, c->uy, c->uz, c->wx, c->wy, c->wz, c->th};
    int r;
    for (int q = 0; q < nf; q++)
        if ((r = download(c, dev[q], h[q]))) return r;
    FILE* f = std::fopen(path, "wb");
    if (!f) { tb_set_error("cannot open %s for writing", path); return TB_ERR_ARG; }
    std::vector<Piece> rec2;
    for (int q = 0; q < nf; q++) rec2.push_back({h[q].data(), h[q].size() * sizeof(cplx)});
    int t32 = t;
    r = write_record(f, {{&t32, 4}});
    if (!r) r = write_record(f, rec2);
    if (std::fclose(f) != 0 && !r) r = TB_ERR_ARG;
    if (r) tb_set_error("write error on %s", path);
    return r;
}

int tb_read_checkpoint(tb_ctx* c, const char* path, int* t) {
    if (!c || !path || !t) { tb_set_error("null argument"); return TB_ERR_ARG; }
    FILE* f = std::fopen(path, "rb");
    if (!f) { tb_set_error("cannot open %s", path); return TB_ERR_ARG; }
    size_t n3 = tb_n3(c);
    const int nf = c->cfg.my_form == 2 ? 7 : 6;
    std::vector<cplx> all(nf * n3);
    int t32 = 0;
    int r = read_record(f, &t32, 4, path);
    if (!r) r = read_record(f, all.data(), all.size() * sizeof(cplx), path);
    std::fclose(f);
    if (r) return r;
    cplx* dev[7] = {c->ux, c->uy, c->uz, c->wx, c->wy, c->wz, c->th};
    for (int q = 0; q < nf; q++)
        TB_CUDA(cudaMemcpyAsync(dev[q], all.data() + q * n3, n3 * sizeof(cplx), cudaMemcpyHostToDevice, c->stream));
    TB_CUDA(cudaStreamSynchronize(c->stream));
    tb_mixed_invalidate(c);
    *t = t32;
    return TB_OK;
}

int tb_write_pert(tb_ctx* c, const char* path) {
    if (!c || !path) { tb_set_error("null argument"); return TB_ERR_ARG; }
    std::vector<cplx> h;
    int r;
    if ((r = download(c, c->ux, h))) return r;
    if (c->cfg.my_form == 0) {   // escreve2 case(0): mode 0 minus the base flow
        size_t n2 = tb_n2(c);
        for (size_t q = 0; q < n2 && q < c->h_uxb.size(); q++) h[q].x -= c->h_uxb[q];
    }
    FILE* f = std::fopen(path, "wb");
    if (!f) { tb_set_error("cannot open %s for writing", path); return TB_ERR_ARG; }
    r = write_record(f, {{h.data(), h.size() * sizeof(cplx)}});
    if (std::fclose(f) != 0 && !r) r = TB_ERR_ARG;
    if (r) tb_set_error("write error on %s", path);
    return r;
}

}  // extern "C"
