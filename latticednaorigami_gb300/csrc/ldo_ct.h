// Working memory of the conserved-topology scaffold regrowth moves, one per
// replica in global memory (allocated only for systems that use them).  It
// holds what the reference keeps in topConstraintPoints::Constraintpoints
// (include/.../top_constraint_points.hpp:221-289), in CTRGRegrowthMCMovetype
// (include/.../rg_movetypes.hpp:73-108) and in the CB movetypes' old/new
// configuration maps, indexed by domain slot instead of hashed by
// (chain, domain): the chains do not change during these moves.  Only the
// replica's move lane touches it, so it needs no layout for coalescing.
#pragma once
#include <stdint.h>
#include "ldo_types.h"

// Scaffold segments of one move (CTRegrowthMCMovetype::select_noncontig_segs
// makes 1 + 2 per stem domain).
#define LDO_CT_MAX_SEGS 64

struct LdoCtEp {
    long long pos;     // packed lattice position
    int16_t cs;        // chain slot of the key (chain, segment)
    int8_t seg;
    int8_t pad;
    int16_t d;         // domain index within its chain
    int16_t pad2;
};

template <class C>
struct LdoCtWork {
    static constexpr int D = C::DCAP;
    static constexpr int EPC = 2 * C::DCAP + 16;   // active endpoints
    static constexpr int EQC = 2 * C::DCAP + 16;   // erased-endpoint queue entries
    static constexpr int FR = 2 * C::KMAX + 8;     // growth frames (staple nesting)

    // ---- Constraintpoints, per domain slot
    int8_t seg[D];            // m_segs (-1: none)
    int16_t gp_to[D];         // m_growthpoints: growth point -> domain grown from it (-1)
    int16_t stem_of[D];       // m_stemdomains: stem domain -> its growth point (-1)
    int16_t inact[D];         // m_inactive_endpoints (-1)
    int8_t ssegs[D][2];       // m_stemd_to_segs
    uint8_t nssegs[D];
    uint8_t in_scaf[D];       // member of the regrown scaffold domains (StapleNetwork::m_scaffold_ds)
    uint8_t in_ds[D];         // member of the current scan's domain stack (m_pot_ds)
    int8_t nseg[D];           // the current scan's segment map
    int8_t sdir[LDO_CT_MAX_SEGS];   // m_domain_to_dir of the scaffold segments (0: unset)
    unsigned long long checked;     // m_checked_staples, by chain slot
    unsigned long long regrow;      // m_regrowth_staples, by chain slot
    // ---- configurations: old (at the start of the move), new, and the
    // one the weight pass restores domain by domain
    long long p_old[D], p_new[D];
    uint8_t o_old[D], o_new[D];
    // ---- regrowth stack (m_d_stack / m_regrow_ds) and recoil-growth state
    int n_rd;
    int16_t rd[D];
    uint8_t catt_q[D], catt_wq[D];
    unsigned long long av_q[D], av_wq[D];   // untried configurations (bit ci of 36)
    double c_open[D];
    // ---- active endpoints in insertion order, and the initial copy
    int n_ep, n_ep0;
    LdoCtEp ep[EPC], ep0[EPC];
    int n_er;                 // m_erased_endpoints
    long long er[EPC];
    int n_eq;                 // m_erased_endpoints_q: level k is eq[eq_off[k] .. eq_off[k + 1])
    int16_t eq_off[D + 2];
    long long eq[EQC];
    // ---- one staple-network scan (StapleNetwork)
    int n_gps, n_iaes, n_nds;
    int16_t gps_a[D], gps_b[D], ia_a[D], ia_b[D], nds[D];
    unsigned long long net_cs;
    int external;
    int16_t scan_cs[C::KMAX + 2], scan_g[C::KMAX + 2], scan_k[C::KMAX + 2];
    // ---- selected segments (CTRegrowthMCMovetype::select_indices /
    // select_noncontig_segs): segment k is seg_dom[seg_off[k] .. seg_off[k + 1])
    int n_segs;
    int16_t seg_off[LDO_CT_MAX_SEGS + 1];
    int16_t seg_dom[D + LDO_CT_MAX_SEGS];
    int8_t seg_dirin[LDO_CT_MAX_SEGS];
    int n_stems;
    int16_t stems[D];
    int16_t pair_off[2 * D + 1];            // paired segment 2i + k of stem i
    int16_t pair_dom[D + LDO_CT_MAX_SEGS];
    int16_t stemq[4 * D];                    // the possible-stem queue
    uint8_t in_sel[D];                       // selected (the `domains` set of select_noncontig_segs)
    // ---- CB growth frames (grow_chain / grow_staple_and_update_endpoints)
    int n_fr;
    int8_t fr_kind[FR];       // 0: list of slots, 1: staple run, 2: staple
    int16_t fr_a[FR], fr_b[FR], fr_n[FR], fr_i[FR];
    int8_t fr_dir[FR];
    int16_t list[D + 1];      // a scaffold list being grown: the stem then a paired segment
    // ---- linker movetypes (LinkerRegrowthMCMovetype, src/transform_movetypes.cpp):
    // the central segment, the domains transformed with it (the segment, then
    // the staples bound to it in chain-index order), the two linkers (each
    // from its central end outwards: lk[0 .. n_lk1) and lk[n_lk1 .. n_lk1 +
    // n_lk2)), the domains that end them (m_linker_endpoints, -1: none), and
    // the trial transformations kept for the Rosenbluth choice
    int n_cen, n_cdom, n_lk1, n_lk2;
    int16_t cen[D], cdom[D], lk[2 * D + 2];
    int16_t lk_end[2];
    int16_t fs_cs[C::KMAX + 2], fs_k[C::KMAX + 2];   // chain scans (find_staples, domains_bound_externally)
    int16_t fs_d[C::KMAX + 2];
    int n_tr;
    long long tr_center[LDO_CT_MAX_TRANSFORMS], tr_disp[LDO_CT_MAX_TRANSFORMS];
    int8_t tr_axis[LDO_CT_MAX_TRANSFORMS], tr_turns[LDO_CT_MAX_TRANSFORMS];
    double tr_bf[LDO_CT_MAX_TRANSFORMS];
    // ---- scalar move state
    int kind;                 // LDO_MV_CT* of the move in progress
    int dir;                  // CTRegrowthMCMovetype::m_dir
    int di, d, ref, stemd, catt, dmax;   // CTRG current domain state
    unsigned long long avail;
    int max_recoils, max_c_attempts;
    double delta_e, weight, weight_new;
    int remove_first[3];
};
