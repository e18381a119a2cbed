// Stand-in for mio (test infrastructure for oracle/_ref): a read-only file mapping with POSIX mmap,
// enough for the reference's out-of-core structure to compile and read.
#pragma once
#include <cstddef>
#include <string>
#include <system_error>
#include <utility>
#include <fcntl.h>
#include <sys/mman.h>
#include <unistd.h>

namespace mio {
class mmap_source {
public:
    mmap_source() = default;
    mmap_source(const mmap_source&) = delete;
    mmap_source& operator=(const mmap_source&) = delete;
    mmap_source(mmap_source&& o) noexcept { swap(o); }
    mmap_source& operator=(mmap_source&& o) noexcept
    {
        if (this != &o) {
            unmap();
            swap(o);
        }
        return *this;
    }
    ~mmap_source() { unmap(); }
    const char* data() const { return m_base ? m_base + m_skew : nullptr; }
    size_t size() const { return m_len; }
    bool is_mapped() const { return m_base != nullptr; }
    void unmap()
    {
        if (m_base)
            ::munmap(const_cast<char*>(m_base), m_len + m_skew);
        m_base = nullptr;
        m_len = m_skew = 0;
    }
    void map(const std::string& path, size_t offset, size_t length, std::error_code& err)
    {
        unmap();
        const int fd = ::open(path.c_str(), O_RDONLY);
        if (fd < 0) {
            err = std::error_code(errno, std::generic_category());
            return;
        }
        const size_t page = size_t(::sysconf(_SC_PAGE_SIZE));
        const size_t aligned = offset / page * page;
        m_skew = offset - aligned;
        void* p = ::mmap(nullptr, length + m_skew, PROT_READ, MAP_SHARED, fd, off_t(aligned));
        ::close(fd);
        if (p == MAP_FAILED) {
            err = std::error_code(errno, std::generic_category());
            m_skew = 0;
            return;
        }
        m_base = static_cast<const char*>(p);
        m_len = length;
    }

private:
    void swap(mmap_source& o)
    {
        std::swap(m_base, o.m_base);
        std::swap(m_len, o.m_len);
        std::swap(m_skew, o.m_skew);
    }
    const char* m_base = nullptr;
    size_t m_len = 0, m_skew = 0;
};
inline mmap_source make_mmap_source(const std::string& path, size_t offset, size_t length, std::error_code& err)
{
    mmap_source m;
    m.map(path, offset, length, err);
    return m;
}
}
