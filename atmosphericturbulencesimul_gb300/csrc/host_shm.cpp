// host_shm.cpp -- the shared-memory image streams of the series command.
//
// The reference publishes frames through its image table's shared images:
// a file /tmp/<name>.im.shm mapped by writer and readers, holding an
// IMAGE_METADATA header followed by the pixels, plus named POSIX
// semaphores <name>_sem00 .. _sem09 and <name>_semlog that readers of that
// format open.  Readers poll cnt0.  This file writes the same layout so the
// reference's readers (and anything built on its CLIcore.h) see our frames.
#include <fcntl.h>
#include <semaphore.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <cerrno>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <ctime>

#include "atmwfs_mkwfs.h"

namespace atmwfs {
void set_error_message(const char* msg);
}

namespace {

// IMAGE_METADATA of src/CLIcore.h:179-203: same members, same C types, so
// the same offsets under this platform's ABI.
struct ImageMetadata {
    char name[80];
    long naxis;
    long size[3];
    long nelement;
    int atype;
    double creation_time;
    double last_access;
    struct timespec wtime;
    int shared;
    int write;
    int status;
    long cnt0;
    long cnt1;
    long NBkw;
};

constexpr const char* kShmDir = "/tmp";   // SHAREDMEMDIR, src/CLIcore.h:45
constexpr int kNumSem = 10;               // COREMOD_memory.c:1855

atmwfs_status err(atmwfs_status s, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    atmwfs::set_error_message(buf);
    return s;
}

}  // namespace

struct atmwfs_shm {
    int fd = -1;
    size_t size = 0;
    ImageMetadata* md = nullptr;
    unsigned char* pix = nullptr;
    size_t frame_bytes = 0;
    sem_t* sem[kNumSem] = {};
    sem_t* semlog = nullptr;
};

extern "C" atmwfs_status atmwfs_shm_create(const char* name, long nx, long ny, int dtype, atmwfs_shm** out)
{
    if (!name || !out || !*name) return err(ATMWFS_ERR_INVALID, "null argument");
    if (strlen(name) >= 80 || strchr(name, '/')) return err(ATMWFS_ERR_INVALID, "bad stream name \"%s\"", name);
    if (nx < 1 || ny < 1) return err(ATMWFS_ERR_INVALID, "bad image size %ld x %ld", nx, ny);
    if (dtype != 3 && dtype != 4) return err(ATMWFS_ERR_INVALID, "data type %d unsupported (3 float, 4 double)", dtype);
    *out = nullptr;
    atmwfs_shm* s = new atmwfs_shm;
    const size_t es = dtype == 3 ? sizeof(float) : sizeof(double);
    s->frame_bytes = (size_t)nx * ny * es;
    // the image's pixels follow the header; no keyword records (NBkw = 0)
    s->size = sizeof(ImageMetadata) + s->frame_bytes;
    char path[256];
    snprintf(path, sizeof path, "%s/%s.im.shm", kShmDir, name);
    s->fd = open(path, O_RDWR | O_CREAT | O_TRUNC, (mode_t)0600);
    if (s->fd == -1) {
        delete s;
        return err(ATMWFS_ERR_IO, "cannot create \"%s\": %s", path, strerror(errno));
    }
    if (ftruncate(s->fd, (off_t)s->size) != 0) {
        close(s->fd);
        delete s;
        return err(ATMWFS_ERR_IO, "cannot size \"%s\": %s", path, strerror(errno));
    }
    void* map = mmap(nullptr, s->size, PROT_READ | PROT_WRITE, MAP_SHARED, s->fd, 0);
    if (map == MAP_FAILED) {
        close(s->fd);
        delete s;
        return err(ATMWFS_ERR_IO, "cannot map \"%s\": %s", path, strerror(errno));
    }
    s->md = (ImageMetadata*)map;
    s->pix = (unsigned char*)map + sizeof(ImageMetadata);
    memset(map, 0, s->size);
    ImageMetadata& md = *s->md;
    snprintf(md.name, sizeof md.name, "%s", name);
    md.naxis = 2;
    md.size[0] = nx;
    md.size[1] = ny;
    md.size[2] = 0;
    md.nelement = nx * ny;
    md.atype = dtype;
    md.shared = 1;
    md.NBkw = 0;
    struct timespec now;
    clock_gettime(CLOCK_REALTIME, &now);
    md.last_access = 1.0 * now.tv_sec + 0.000000001 * now.tv_nsec;
    md.creation_time = md.last_access;
    md.write = 0;
    md.cnt0 = 0;
    md.cnt1 = 0;
    // semaphores: <name>_semlog, and <name>_sem00.._sem09 opened or created
    // at 0 with stale higher-numbered ones removed (COREMOD_memory.c:1555-1562, 4071-4125)
    char sname[160];
    snprintf(sname, sizeof sname, "%s_semlog", name);
    sem_unlink(sname);
    s->semlog = sem_open(sname, O_CREAT, 0644, 0);
    if (s->semlog == SEM_FAILED) s->semlog = nullptr;
    for (int k = kNumSem; k < 100; k++) {
        snprintf(sname, sizeof sname, "%s_sem%02d", name, k);
        sem_unlink(sname);
    }
    for (int k = 0; k < kNumSem; k++) {
        snprintf(sname, sizeof sname, "%s_sem%02d", name, k);
        sem_t* p = sem_open(sname, 0);
        if (p == SEM_FAILED) p = sem_open(sname, O_CREAT, 0644, 0);
        s->sem[k] = p == SEM_FAILED ? nullptr : p;
    }
    *out = s;
    return ATMWFS_OK;
}

extern "C" atmwfs_status atmwfs_shm_write(atmwfs_shm* s, const void* frame, int bump)
{
    if (!s || !frame) return err(ATMWFS_ERR_INVALID, "null argument");
    volatile ImageMetadata* md = s->md;
    if (bump) md->write = 1;
    memcpy(s->pix, frame, s->frame_bytes);
    if (bump) {
        __atomic_thread_fence(__ATOMIC_RELEASE);
        md->cnt0 = md->cnt0 + 1;
        md->write = 0;
    }
    return ATMWFS_OK;
}

extern "C" void atmwfs_shm_close(atmwfs_shm* s)
{
    if (!s) return;
    for (sem_t* p : s->sem)
        if (p) sem_close(p);
    if (s->semlog) sem_close(s->semlog);
    if (s->md) munmap(s->md, s->size);
    if (s->fd >= 0) close(s->fd);
    delete s;
}

extern "C" atmwfs_status atmwfs_shm_semwait(const char* name, long index, double timeout_s)
{
    if (!name || index < 0 || index > 99) return err(ATMWFS_ERR_INVALID, "bad semaphore request");
    char sname[160];
    snprintf(sname, sizeof sname, "%s_sem%02ld", name, index);
    sem_t* p = sem_open(sname, 0);
    if (p == SEM_FAILED) return err(ATMWFS_ERR_INVALID, "image %s semaphore # %ld does not exist", name, index);
    int r;
    if (timeout_s > 0) {
        struct timespec t;
        clock_gettime(CLOCK_REALTIME, &t);
        const double whole = floor(timeout_s);
        t.tv_sec += (time_t)whole;
        t.tv_nsec += (long)((timeout_s - whole) * 1e9);
        if (t.tv_nsec >= 1000000000L) {
            t.tv_sec++;
            t.tv_nsec -= 1000000000L;
        }
        do r = sem_timedwait(p, &t);
        while (r != 0 && errno == EINTR);
    } else {
        do r = sem_wait(p);
        while (r != 0 && errno == EINTR);
    }
    const int e = errno;
    sem_close(p);
    if (r != 0)
        return e == ETIMEDOUT ? err(ATMWFS_ERR_TIMEOUT, "semaphore %s: no post within %g s", sname, timeout_s)
                              : err(ATMWFS_ERR_IO, "semaphore %s: %s", sname, strerror(e));
    return ATMWFS_OK;
}
