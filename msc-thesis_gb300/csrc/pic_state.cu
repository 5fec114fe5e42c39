// pic_state.cu -- state files (checkpoint / resume).
//
// Layout (little-endian):
//   "PICSTATE" u32 version=1
//   i32 nx, ny; f64 Lx, Ly, dt, eps0; i32 nspecies
//   i64 step; u64 mcc_pass, dsmc_pass
//   per species: i64 n; i32 flags, q_int; f64 q, m
//   per species, in storage order: i32 cell[n]; f32 ox[n], oy[n], vx[n], vy[n];
//     f32 vz[n] when PIC_SPECIES_HAS_VZ; u32 pid[n]
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "pic_internal.cuh"

namespace {

const char MAGIC[8] = {'P', 'I', 'C', 'S', 'T', 'A', 'T', 'E'};
const uint32_t VERSION = 1;

struct File {
    FILE *f = nullptr;
    ~File()
    {
        if (f) fclose(f);
    }
};

template <class T> bool put(FILE *f, const T &v) { return fwrite(&v, sizeof(T), 1, f) == 1; }
template <class T> bool get(FILE *f, T &v) { return fread(&v, sizeof(T), 1, f) == 1; }

pic_status io_fail(const std::string &what)
{
    pic::set_error(what);
    return PIC_ERR_INVALID_ARG;
}

// device array -> file through a host buffer
pic_status dump(FILE *f, const void *dev, size_t bytes, std::vector<char> &buf)
{
    buf.resize(bytes);
    if (bytes) PIC_CUDA(cudaMemcpy(buf.data(), dev, bytes, cudaMemcpyDeviceToHost));
    if (bytes && fwrite(buf.data(), 1, bytes, f) != bytes) return io_fail("pic_save: write failed");
    return PIC_OK;
}

// A loaded species must be one the kernels can take: cells on the grid or
// -1 (an empty slot, left by an ionisation that overflowed the capacity),
// offsets in [0, 1), finite velocities, ids a permutation of 0..n-1.
std::string check_species(const char *p, size_t n, bool has_vz, int nx, int ny)
{
    std::vector<int32_t> cell(n);
    std::vector<float> v(n);
    std::vector<uint32_t> pid(n);
    memcpy(cell.data(), p, n * 4);
    for (size_t i = 0; i < n; ++i) {
        const int32_t c = cell[i];
        if (c != -1 && (c < 0 || (c & 0xFFFF) >= nx || (c >> 16) >= ny))
            return "cell index off the grid";
    }
    for (int a = 1; a < (has_vz ? 6 : 5); ++a) {
        memcpy(v.data(), p + (size_t)a * n * 4, n * 4);
        for (size_t i = 0; i < n; ++i) {
            if (cell[i] == -1) continue;
            const float x = v[i];
            if (a <= 2 ? !(x >= 0.f && x < 1.f) : !std::isfinite(x))
                return a <= 2 ? "cell offset outside [0, 1)" : "non-finite velocity";
        }
    }
    memcpy(pid.data(), p + (size_t)(has_vz ? 6 : 5) * n * 4, n * 4);
    std::vector<char> seen(n, 0);
    for (size_t i = 0; i < n; ++i) {
        if (pid[i] >= n || seen[pid[i]]) return "particle ids are not a permutation";
        seen[pid[i]] = 1;
    }
    return "";
}

}  // namespace

extern "C" pic_status pic_save(pic_handle *h, const char *path)
{
    if (!h || !path) return io_fail("pic_save: null argument");
    PIC_CUDA(cudaSetDevice(h->device));
    PIC_CUDA(cudaStreamSynchronize(h->stream));
    pic::DevState st;
    PIC_CUDA(cudaMemcpy(&st, h->dev, sizeof st, cudaMemcpyDeviceToHost));
    File F;
    F.f = fopen(path, "wb");
    if (!F.f) return io_fail(std::string("pic_save: cannot open ") + path);
    FILE *f = F.f;
    const pic_config &c = h->cfg;
    bool ok = fwrite(MAGIC, 1, 8, f) == 8 && put(f, VERSION) && put(f, c.nx) && put(f, c.ny) &&
              put(f, c.Lx) && put(f, c.Ly) && put(f, c.dt) && put(f, c.eps0) &&
              put(f, c.nspecies) && put(f, st.step) && put(f, st.mcc_pass) &&
              put(f, st.dsmc_pass);
    for (int s = 0; ok && s < c.nspecies; ++s) {
        const pic_species_desc &D = c.species[s];
        ok = put(f, st.n[s]) && put(f, D.flags) && put(f, D.q_int) && put(f, D.q) && put(f, D.m);
    }
    if (!ok) return io_fail("pic_save: write failed");
    std::vector<char> buf;
    for (int s = 0; s < c.nspecies; ++s) {
        const pic::SpeciesBuf &B = h->sp[s];
        const size_t n = (size_t)st.n[s];
        PIC_TRY(dump(f, B.cell[0], n * 4, buf));
        PIC_TRY(dump(f, B.ox[0], n * 4, buf));
        PIC_TRY(dump(f, B.oy[0], n * 4, buf));
        PIC_TRY(dump(f, B.vx[0], n * 4, buf));
        PIC_TRY(dump(f, B.vy[0], n * 4, buf));
        if (B.vz[0]) PIC_TRY(dump(f, B.vz[0], n * 4, buf));
        PIC_TRY(dump(f, B.pid[0], n * 4, buf));
    }
    return fflush(f) == 0 ? PIC_OK : io_fail("pic_save: write failed");
}

namespace pic {
pic_status handle_reload(pic_handle *h, const long long *n, long long step,
                         unsigned long long mcc_pass, unsigned long long dsmc_pass);
}

extern "C" pic_status pic_load(pic_handle *h, const char *path)
{
    if (!h || !path) return io_fail("pic_load: null argument");
    PIC_CUDA(cudaSetDevice(h->device));
    PIC_CUDA(cudaStreamSynchronize(h->stream));
    File F;
    F.f = fopen(path, "rb");
    if (!F.f) return io_fail(std::string("pic_load: cannot open ") + path);
    FILE *f = F.f;
    char magic[8];
    uint32_t ver = 0;
    int nx, ny, ns;
    double Lx, Ly, dt, eps0;
    long long step;
    unsigned long long mp, dp;
    if (fread(magic, 1, 8, f) != 8 || memcmp(magic, MAGIC, 8) != 0 || !get(f, ver) || ver != VERSION)
        return io_fail("pic_load: not a state file of this version");
    if (!get(f, nx) || !get(f, ny) || !get(f, Lx) || !get(f, Ly) || !get(f, dt) || !get(f, eps0) ||
        !get(f, ns) || !get(f, step) || !get(f, mp) || !get(f, dp))
        return io_fail("pic_load: file truncated");
    const pic_config &c = h->cfg;
    if (nx != c.nx || ny != c.ny || Lx != c.Lx || Ly != c.Ly || ns != c.nspecies)
        return io_fail("pic_load: grid or species count differs from the handle's");
    // a resumed run continues bit for bit only under the same step and
    // permittivity, so a file written under others is refused
    if (dt != c.dt || eps0 != c.eps0)
        return io_fail("pic_load: time step or permittivity differs from the handle's");
    long long n[PIC_MAX_SPECIES] = {0, 0, 0, 0};
    for (int s = 0; s < ns; ++s) {
        int flags, q_int;
        double q, m;
        if (!get(f, n[s]) || !get(f, flags) || !get(f, q_int) || !get(f, q) || !get(f, m))
            return io_fail("pic_load: file truncated");
        const pic_species_desc &D = c.species[s];
        if (n[s] < 0 || n[s] > D.capacity || flags != D.flags || q_int != D.q_int || q != D.q ||
            m != D.m)
            return io_fail("pic_load: species " + std::to_string(s) +
                           " does not fit the handle (count, flags, charge or mass)");
    }
    // read and check everything before the handle is touched, so that a bad
    // file leaves it as it was
    std::vector<std::vector<char>> body(ns);
    for (int s = 0; s < ns; ++s) {
        const size_t m = (size_t)n[s];
        const int arrays = h->sp[s].vz[0] ? 7 : 6;
        body[s].resize(m * 4 * arrays);
        if (m && fread(body[s].data(), 1, body[s].size(), f) != body[s].size())
            return io_fail("pic_load: file truncated");
        const std::string bad = check_species(body[s].data(), m, arrays == 7, nx, ny);
        if (!bad.empty()) return io_fail("pic_load: species " + std::to_string(s) + ": " + bad);
    }
    if (fgetc(f) != EOF) return io_fail("pic_load: trailing bytes after the last species");
    for (int s = 0; s < ns; ++s) {
        pic::SpeciesBuf &B = h->sp[s];
        const size_t m = (size_t)n[s];
        const char *p = body[s].data();
        void *dst[7] = {B.cell[0], B.ox[0], B.oy[0], B.vx[0], B.vy[0], B.vz[0], B.pid[0]};
        for (int a = 0; a < 7; ++a) {
            if (!dst[a]) continue;
            if (m) PIC_CUDA(cudaMemcpy(dst[a], p, m * 4, cudaMemcpyHostToDevice));
            p += m * 4;
        }
    }
    return pic::handle_reload(h, n, step, mp, dp);
}
