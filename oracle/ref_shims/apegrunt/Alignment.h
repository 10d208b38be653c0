/* Test-oracle stand-in for the parts of apegrunt (an absent SuperDCA
 * submodule, github.com/santeripuranen/apegrunt, no pinned commit) that the
 * SuperDCA solve headers touch: the 4-state "triallelic" state type, 16-locus
 * state blocks with per-block unique patterns ("block storage" and "block
 * accounting"), sequence multiplicities and frequencies, and a packed
 * lower-triangular Hamming distance matrix.  Written from the call sites in
 * SuperDCA/include/plmDCA_objective.hpp:56-121 and
 * SuperDCA/include/plmDCA_optimizer_parameters.hpp:39-98,297-347.
 *
 * Only oracle/ref_golden.cpp includes this, to compile the reference's own
 * headers into oracle/_ref for golden vectors.  Unknown apegrunt semantics are
 * fixed here as: GAP is state 3; the distance counts loci whose codes differ;
 * patterns are listed per block in order of first occurrence. */
#pragma once

#include <array>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <map>
#include <memory>
#include <new>
#include <tuple>
#include <vector>

namespace boost { using std::get; }

namespace apegrunt {

enum triallelic_state_t : std::uint8_t { TRI_0 = 0, TRI_1 = 1, TRI_2 = 2, GAP = 3 };

template <typename StateT> struct number_of_states;
template <> struct number_of_states<triallelic_state_t> { enum { value = 4, N = 4 }; };

constexpr std::size_t StateBlock_size = 16;

template <typename StateT, std::size_t Size>
struct State_block {
    std::array<StateT, Size> s{};
    StateT operator[](std::size_t i) const { return s[i]; }
};

namespace memory {
template <typename T>
struct AlignedAllocator {
    using value_type = T;
    AlignedAllocator() = default;
    template <typename U> AlignedAllocator(const AlignedAllocator<U> &) {}
    T *allocate(std::size_t n)
    {
        void *p = nullptr;
        if (posix_memalign(&p, 64, n * sizeof(T) + 64) != 0) throw std::bad_alloc();
        return static_cast<T *>(p);
    }
    void deallocate(T *p, std::size_t) { std::free(p); }
    template <typename U> struct rebind { using other = AlignedAllocator<U>; };
    bool operator==(const AlignedAllocator &) const { return true; }
    bool operator!=(const AlignedAllocator &) const { return false; }
};
} // namespace memory

struct Sequence {
    std::vector<std::uint8_t> states;
    std::size_t mult = 1;
    std::array<std::size_t, 4> freq{};
    std::size_t size() const { return states.size(); }
    std::size_t multiplicity() const { return mult; }
    const std::array<std::size_t, 4> &frequencies() const { return freq; }
    triallelic_state_t operator[](std::size_t i) const { return triallelic_state_t(states[i]); }
};
using Sequence_ptr = std::shared_ptr<Sequence>;

template <typename StateT>
class Alignment {
public:
    using block_t = State_block<StateT, StateBlock_size>;
    using block_storage_t = std::vector<std::vector<block_t>>;
    using block_accounting_t = std::vector<std::vector<std::vector<std::size_t>>>;

    Alignment(const std::uint8_t *states, std::size_t N, std::size_t L, const double *mult)
        : m_L(L)
    {
        for (std::size_t i = 0; i < N; ++i) {
            auto s = std::make_shared<Sequence>();
            s->states.assign(states + i * L, states + (i + 1) * L);
            s->mult = mult ? std::size_t(mult[i]) : 1;
            for (auto c : s->states) s->freq[c]++;
            m_seqs.push_back(s);
        }
        build_blocks();
        build_distances();
    }

    std::size_t n_loci() const { return m_L; }
    std::size_t size() const { return m_seqs.size(); }
    std::size_t effective_size() const
    {
        std::size_t n = 0;
        for (auto &s : m_seqs) n += s->mult;
        return n;
    }
    struct Subscript {
        const std::vector<Sequence_ptr> *seqs;
        const Sequence_ptr &operator[](std::size_t i) const { return (*seqs)[i]; }
    };
    Subscript subscript_proxy() const { return Subscript{&m_seqs}; }
    std::vector<Sequence_ptr>::const_iterator begin() const { return m_seqs.begin(); }
    std::vector<Sequence_ptr>::const_iterator end() const { return m_seqs.end(); }
    std::shared_ptr<block_storage_t> get_block_storage() const { return m_blocks; }
    std::shared_ptr<block_accounting_t> get_block_accounting() const { return m_accounting; }
    std::shared_ptr<std::vector<std::size_t>> distance_matrix() const { return m_dist; }

private:
    void build_blocks()
    {
        const std::size_t nb = (m_L + StateBlock_size - 1) / StateBlock_size;
        m_blocks = std::make_shared<block_storage_t>(nb);
        m_accounting = std::make_shared<block_accounting_t>(nb);
        for (std::size_t b = 0; b < nb; ++b) {
            std::map<std::vector<std::uint8_t>, std::size_t> index;
            for (std::size_t i = 0; i < m_seqs.size(); ++i) {
                block_t blk;
                std::vector<std::uint8_t> key;
                for (std::size_t p = 0; p < StateBlock_size; ++p) {
                    const std::size_t n = b * StateBlock_size + p;
                    const std::uint8_t c = n < m_L ? m_seqs[i]->states[n] : 0;
                    blk.s[p] = StateT(c);
                    key.push_back(c);
                }
                auto it = index.find(key);
                if (it == index.end()) {
                    it = index.emplace(key, (*m_blocks)[b].size()).first;
                    (*m_blocks)[b].push_back(blk);
                    (*m_accounting)[b].emplace_back();
                }
                (*m_accounting)[b][it->second].push_back(i);
            }
        }
    }
    void build_distances()
    {
        const std::size_t N = m_seqs.size();
        m_dist = std::make_shared<std::vector<std::size_t>>(N * (N - 1) / 2 + 1, 0);
        for (std::size_t i = 1; i < N; ++i)
            for (std::size_t j = 0; j < i; ++j) {
                std::size_t d = 0;
                for (std::size_t n = 0; n < m_L; ++n) d += m_seqs[i]->states[n] != m_seqs[j]->states[n];
                (*m_dist)[i * (i - 1) / 2 + j] = d;
            }
    }

    std::size_t m_L;
    std::vector<Sequence_ptr> m_seqs;
    std::shared_ptr<block_storage_t> m_blocks;
    std::shared_ptr<block_accounting_t> m_accounting;
    std::shared_ptr<std::vector<std::size_t>> m_dist;
};

template <typename StateT> using Alignment_ptr = std::shared_ptr<Alignment<StateT>>;

template <typename StateT>
auto begin(const std::shared_ptr<Alignment<StateT>> &a) { return a->begin(); }
template <typename StateT>
auto end(const std::shared_ptr<Alignment<StateT>> &a) { return a->end(); }

template <typename T>
auto cbegin(const std::shared_ptr<std::vector<T>> &v) { return v->cbegin(); }
template <typename T>
auto cend(const std::shared_ptr<std::vector<T>> &v) { return v->cend(); }

template <typename StateT>
std::vector<std::tuple<std::size_t, Sequence_ptr>> zip_range(const std::vector<std::size_t> &w,
                                                             const Alignment<StateT> &a)
{
    std::vector<std::tuple<std::size_t, Sequence_ptr>> out;
    auto ali = a.subscript_proxy();
    for (std::size_t i = 0; i < w.size(); ++i) out.emplace_back(w[i], ali[i]);
    return out;
}

} // namespace apegrunt
