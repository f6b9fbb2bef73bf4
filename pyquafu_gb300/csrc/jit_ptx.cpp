// PTX generator of circuit-specialised tile passes (see jit.h).
//
// The emitted kernel is the tile pass of device.cuh (k_pass) / adjoint.cuh
// (k_pass2) with the plan's steps unrolled: the persistent tile loop, the
// cp.async staging of a tile into swizzled shared memory, for every
// register round the loads, the gate arithmetic and the stores, all with
// compile-time register indices, and two-target dense gates as
// shared-memory steps over the tile.  The gate arithmetic follows the policy
// primitives of policy.cuh operation for operation (mul.rn / fma.rn / add.rn,
// no contraction), so the specialised passes compute what the interpreting
// kernels compute.  Register permutations (X, SWAP, Y, quarter turns) are
// renames of PTX virtual registers and cost no instruction.
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "jit.h"
#include "qfvm_gb300.h"

namespace qsv {
namespace {

std::string fmt(const char* f, ...) {
    char buf[640];
    va_list ap;
    va_start(ap, f);
    vsnprintf(buf, sizeof buf, f, ap);
    va_end(ap);
    return buf;
}

struct Cx {
    std::string x, y;
};
bool same(const Cx& a, const Cx& b) { return a.x == b.x && a.y == b.y; }

class Gen {
   public:
    Gen(const HostPlan& hp, int pi, const JitShape& sh)
        : hp_(hp), pd_(hp.passes[pi]), sh_(sh) {
        f64_ = hp.arith == QFVM_C128;
        ds_ = hp.arith == QFVM_C128_DS;
        ft_ = f64_ ? "f64" : "f32";
        es_ = (f64_ || ds_) ? 16 : 8;
        cb_ = (f64_ || ds_) ? 8 : 4;
        T_ = hp.T;
        R_ = hp.R;
        NT_ = 1 << (T_ - R_);
        NA_ = 1 << R_;
        NW_ = NT_ / 32;
        PER_ = (1 << T_) / NT_;
        NS_ = sh.nstates;
        np_ = NS_ == 2 ? pd_.nprobe : 0;
        padu_ = 16u / static_cast<uint32_t>(es_);
        H_ = T_ - TILE_RUN_BITS;
        RUNS_ = 1 << H_;
        runB_ = static_cast<uint32_t>(es_) << TILE_RUN_BITS;
        tileB_ = tile_elems(T_, es_) * static_cast<uint32_t>(es_);
        slotB_ = tileB_ * NS_;
        bc_ = sh.bounds != 0;
        // double-single plans chained in float-pair format: every pass but
        // the first reads float pairs, every pass but the last writes them
        in_pair_ = ds_ && sh.chain && pi > 0;
        out_pair_ = ds_ && sh.chain && pi + 1 < static_cast<int>(hp.passes.size());
        bulk_out_ = !ds_ || out_pair_;
        if (sh.pcoef) coef_range(&cmin_, &cmax_);
        pc_ = sh.pcoef && cmax_ > cmin_ && blob_bytes() <= kMaxBlob;
    }

    // Coefficient pool entries the pass's operations read: [lo, hi).
    void coef_range(uint32_t* lo, uint32_t* hi) const {
        *lo = ~0u;
        *hi = 0;
        for (int si = 0; si < pd_.step_count; ++si) {
            const StepDesc& sd = hp_.steps[pd_.step_begin + si];
            for (int oi = 0; oi < sd.op_count; ++oi) {
                const KOp& o = hp_.ops[sd.op_begin + oi];
                int n = 0;
                switch (o.kind) {
                    case K_DENSE: n = 8; break;
                    case K_REAL: case K_DIAG: n = 4; break;
                    case K_RX: n = 2; break;
                    case K_DIAGR: n = 2 * NA_; break;
                    case K_DENSE2: n = 32; break;
                    case K_PROBE: n = 1; break;
                    default: break;
                }
                if (n == 0) continue;
                if (o.coef < *lo) *lo = o.coef;
                if (o.coef + n > *hi) *hi = o.coef + n;
            }
        }
        if (*hi == 0) *lo = 0;
    }
    uint32_t blob_bytes() const { return ((cmax_ - cmin_) * cb_ + 15u) / 16u * 16u; }

    bool param_coefs() const { return pc_; }
    bool in_pairs() const { return in_pair_; }
    bool out_pairs() const { return out_pair_; }
    uint32_t cmin() const { return cmin_; }
    uint32_t cmax() const { return cmax_; }


    bool supported(std::string* why) const {
        if (hp_.arith != QFVM_C64 && hp_.arith != QFVM_C128 && hp_.arith != QFVM_C128_DS)
            return no(why, "arithmetic without a generator");
        if (pd_.type != PASS_TILE) return no(why, "not a tile pass");
        if (pd_.L != TILE_RUN_BITS || pd_.H != T_ - TILE_RUN_BITS) return no(why, "tile without 32-amplitude runs");
        if (T_ - R_ < 6 || T_ > 13 || R_ < 1 || R_ > 5) return no(why, "tile shape out of range");
        if (np_ > NT_ || np_ > MAX_PASS_PROBES) return no(why, "too many probes");
        for (int si = 0; si < pd_.step_count; ++si) {
            const StepDesc& sd = hp_.steps[pd_.step_begin + si];
            for (int oi = 0; oi < sd.op_count; ++oi) {
                const KOp& o = hp_.ops[sd.op_begin + oi];
                if (sd.type == STEP_SMEM) {
                    if (o.kind != K_DENSE2) return no(why, "shared-memory step kind without a generator");
                    continue;
                }
                switch (o.kind) {
                    case K_DENSE: case K_REAL: case K_RX: case K_DIAG: case K_X: case K_Y: case K_SWAP: case K_HAD:
                        break;
                    case K_DIAGR:
                        if (o.k != R_) return no(why, "merged diagonal of another register count");
                        break;
                    case K_PROBE:
                        if (NS_ != 2) return no(why, "probe in a one-state pass");
                        break;
                    default: return no(why, "operation kind without a generator");
                }
            }
        }
        return true;
    }

    std::string emit(const std::string& entry) {
        prologue();
        tile_loop();
        std::string out;
        out += "//\n// circuit-specialised tile pass\n//\n.version 9.0\n.target sm_103a\n.address_size 64\n\n";
        out += ".extern .shared .align 16 .b8 qsv_dsm[];\n\n";
        out += ".visible .entry " + entry + "(\n";
        out += "\t.param .u64 p_psi,\n\t.param .u64 p_lam,\n\t.param .u64 p_ntiles,\n\t.param .u64 p_coef,\n";
        out += "\t.param .u64 p_cstride,\n\t.param .u32 p_ishift,\n\t.param .u64 p_active,\n";
        out += "\t.param .u32 p_per_tile,\n\t.param .u64 p_partial,\n\t.param .u64 p_status,\n";
        out += "\t.param .u64 p_wait_ns,\n\t.param .u32 p_extra_tx";
        if (pc_) out += fmt(",\n\t.param .align 16 .b8 p_cblob[%u]", blob_bytes());
        out += "\n)\n";
        out += fmt(".maxntid %d, 1, 1\n.minnctapersm %d\n{\n", NT_, sh_.minb < 1 ? 1 : sh_.minb);
        out += fmt("\t.reg .pred %%p<%d>;\n\t.reg .b16 %%h<%d>;\n\t.reg .b32 %%r<%d>;\n\t.reg .b64 %%rd<%d>;\n",
                   np_reg_ + 1, nh_ + 1, nr_ + 1, nrd_ + 1);
        out += fmt("\t.reg .%s %%a<%d>;\n\t.reg .f64 %%d<%d>;\n\n", ft_, na_ + 1, nd_ + 1);
        out += body_;
        out += "}\n";
        return out;
    }

   private:
    static bool no(std::string* why, const char* m) {
        if (why) *why = m;
        return false;
    }

    // ---------------------------------------------------------------- emission
    std::string R32() { return "%r" + std::to_string(nr_++); }
    std::string R64() { return "%rd" + std::to_string(nrd_++); }
    std::string H16() { return "%h" + std::to_string(nh_++); }
    std::string P() { return "%p" + std::to_string(np_reg_++); }
    std::string A() { return "%a" + std::to_string(na_++); }
    std::string D() { return "%d" + std::to_string(nd_++); }
    std::string L() { return "$L" + std::to_string(nl_++); }
    void I(const std::string& s) { Iraw(bc_ ? checked(s) : s); }
    // a comment line in the emitted PTX (marks what the following
    // instructions do, for readers of the generated code)
    void note(const std::string& s) {
        body_ += "\t// ";
        body_ += s;
        body_ += '\n';
    }
    void Iraw(const std::string& s) {
        body_ += '\t';
        body_ += s;
        body_ += ";\n";
    }

    // Bounds-checked builds: a shared-memory access, a global store or a bulk
    // copy is guarded by a check of its address range against the dynamic
    // shared memory / the states; outside, the access is skipped and the
    // thread writes QFVM_ERR_BOUNDS to the status word.  Returns the access,
    // predicated on the check (and on its own predicate, if it had one).
    std::string checked(const std::string& ins) {
        std::string pred, body = ins;
        if (!ins.empty() && ins[0] == '@') {
            const size_t sp = ins.find(' ');
            pred = ins.substr(1, sp - 1);
            body = ins.substr(sp + 1);
        }
        auto starts = [&](const char* p) { return body.compare(0, std::strlen(p), p) == 0; };
        const bool shared = starts("ld.shared") || starts("st.shared");
        const bool gstore = starts("st.global.cs");
        const bool bload = starts("cp.async.bulk.shared::cluster.global");
        const bool bstore = starts("cp.async.bulk.global.shared::cta");
        if (!shared && !gstore && !bload && !bstore) return ins;
        // address operands [reg] or [reg+imm], in order
        std::vector<std::pair<std::string, uint64_t>> ad;
        for (size_t a = body.find('['); a != std::string::npos; a = body.find('[', a + 1)) {
            const size_t e = body.find(']', a);
            const std::string op = body.substr(a + 1, e - a - 1);
            const size_t plus = op.find('+');
            if (plus == std::string::npos) ad.push_back({op, 0});
            else ad.push_back({op.substr(0, plus), std::stoull(op.substr(plus + 1))});
        }
        uint32_t size = runB_;
        if (shared || gstore) {
            const std::string opc = body.substr(0, body.find(' '));  // e.g. ld.shared.v2.f64
            const int w = opc.find(".v4.") != std::string::npos ? 4 : (opc.find(".v2.") != std::string::npos ? 2 : 1);
            const bool b8 = opc.size() >= 2 && opc.compare(opc.size() - 2, 2, "64") == 0;
            size = static_cast<uint32_t>(w * (b8 ? 8 : 4));
        }
        std::vector<std::string> oks;
        auto shared_ok = [&](const std::pair<std::string, uint64_t>& a) {
            std::string ea = R32(), eb = R32(), q = P(), ok = P();
            Iraw(fmt("add.u32 %s, %s, %llu", ea.c_str(), a.first.c_str(), static_cast<unsigned long long>(a.second)));
            Iraw(fmt("setp.ge.u32 %s, %s, %s", q.c_str(), ea.c_str(), smb_.c_str()));
            Iraw(fmt("add.u32 %s, %s, %u", eb.c_str(), ea.c_str(), size));
            Iraw(fmt("setp.le.and.u32 %s, %s, %s, %s", ok.c_str(), eb.c_str(), smend_.c_str(), q.c_str()));
            oks.push_back(ok);
        };
        auto global_ok = [&](const std::pair<std::string, uint64_t>& a) {
            std::string ga = R64(), gb = R64(), any = P();
            Iraw(fmt("add.s64 %s, %s, %llu", ga.c_str(), a.first.c_str(), static_cast<unsigned long long>(a.second)));
            Iraw(fmt("add.s64 %s, %s, %u", gb.c_str(), ga.c_str(), size));
            for (int st = 0; st < NS_; ++st) {
                std::string q = P(), ok = P();
                Iraw(fmt("setp.ge.u64 %s, %s, %s", q.c_str(), ga.c_str(), stg_[st].c_str()));
                Iraw(fmt("setp.le.and.u64 %s, %s, %s, %s", ok.c_str(), gb.c_str(), gend_[st].c_str(), q.c_str()));
                if (st == 0) Iraw(fmt("mov.pred %s, %s", any.c_str(), ok.c_str()));
                else Iraw(fmt("or.pred %s, %s, %s", any.c_str(), any.c_str(), ok.c_str()));
            }
            oks.push_back(any);
        };
        if (shared) shared_ok(ad[0]);
        if (gstore) global_ok(ad[0]);
        if (bload) {
            shared_ok(ad[0]);
            global_ok(ad[1]);
        }
        if (bstore) {
            global_ok(ad[0]);
            shared_ok(ad[1]);
        }
        std::string ok = oks[0];
        for (size_t k = 1; k < oks.size(); ++k) {
            std::string n = P();
            Iraw(fmt("and.pred %s, %s, %s", n.c_str(), ok.c_str(), oks[k].c_str()));
            ok = n;
        }
        std::string bad = P();
        Iraw(fmt("not.pred %s, %s", bad.c_str(), ok.c_str()));
        if (!pred.empty()) {
            std::string both = P(), bad2 = P();
            Iraw(fmt("and.pred %s, %s, %s", both.c_str(), ok.c_str(), pred.c_str()));
            Iraw(fmt("and.pred %s, %s, %s", bad2.c_str(), bad.c_str(), pred.c_str()));
            ok = both;
            bad = bad2;
        }
        std::string old = R32();  // the first error recorded stays
        Iraw(fmt("@%s atom.global.cas.b32 %s, [%s], 0, %d", bad.c_str(), old.c_str(), status_.c_str(),
                 static_cast<int>(QFVM_ERR_BOUNDS)));
        return "@" + ok + " " + body;
    }
    void lab(const std::string& l) { body_ += l + ":\n"; }

    // Amplitude-type arithmetic (policy.cuh: mul / madd / add / neg).  A real
    // value is a register name, or for double-single "high|low" (two f32).
    static std::pair<std::string, std::string> hl(const std::string& v) {
        const size_t k = v.find('|');
        return {v.substr(0, k), v.substr(k + 1)};
    }
    std::string f32op(const char* op, const std::string& a, const std::string& b) {
        std::string d = A();
        I(fmt("%s.rn.f32 %s, %s, %s", op, d.c_str(), a.c_str(), b.c_str()));
        return d;
    }
    std::string f32fma(const std::string& a, const std::string& b, const std::string& c) {
        std::string d = A();
        I(fmt("fma.rn.f32 %s, %s, %s, %s", d.c_str(), a.c_str(), b.c_str(), c.c_str()));
        return d;
    }
    std::string f32neg(const std::string& a) {
        std::string d = A();
        I(fmt("neg.f32 %s, %s", d.c_str(), a.c_str()));
        return d;
    }
    // Double-single values inside a pass are float pairs (h, l) that need not
    // be renormalised: h + l is the value, and |l| stays below a few units in
    // the last place of the operands that made it, so every operation's
    // absolute error stays near 2^-46 of its operands' magnitudes.  Pairs are
    // renormalised (TwoSum) only where the FP64 conversion needs |l| <= |h|.
    // a + b: TwoSum of the high parts, low parts and error summed
    std::string ds_add(const std::string& a, const std::string& b) {
        auto [ah, al] = hl(a);
        auto [bh, bl] = hl(b);
        const std::string sh = f32op("add", ah, bh);
        const std::string v = f32op("sub", sh, ah);
        std::string e = f32op("add", f32op("sub", ah, f32op("sub", sh, v)), f32op("sub", bh, v));
        e = f32op("add", e, f32op("add", al, bl));
        return sh + "|" + e;
    }
    // (h, l) -> the same value with |l| <= ulp(h) / 2 (TwoSum: exact for any pair)
    std::string ds_norm(const std::string& a) {
        auto [h, l] = hl(a);
        const std::string s = f32op("add", h, l);
        const std::string v = f32op("sub", s, h);
        const std::string e = f32op("add", f32op("sub", h, f32op("sub", s, v)), f32op("sub", l, v));
        return s + "|" + e;
    }
    std::string ds_mul_raw(const std::string& c, const std::string& x) {
        auto [ch, cl] = hl(c);
        auto [xh, xl] = hl(x);
        const std::string p = f32op("mul", ch, xh);
        std::string e = f32fma(ch, xh, f32neg(p));
        e = f32fma(ch, xl, e);
        e = f32fma(cl, xh, e);
        return p + "|" + e;
    }
    std::string mul(const std::string& c, const std::string& x) {
        if (ds_) return ds_mul_raw(c, x);
        std::string d = A();
        I(fmt("mul.rn.%s %s, %s, %s", ft_, d.c_str(), c.c_str(), x.c_str()));
        return d;
    }
    std::string fma(const std::string& c, const std::string& x, const std::string& acc) {
        if (ds_) return ds_add(acc, ds_mul_raw(c, x));
        std::string d = A();
        I(fmt("fma.rn.%s %s, %s, %s, %s", ft_, d.c_str(), c.c_str(), x.c_str(), acc.c_str()));
        return d;
    }
    // sum of c_i * x_i.  FP64 / FP32: mul then fma in order (the same
    // roundings as the nested mul / fma form).  Double-single: every product
    // split exactly (FMA TwoProd), the products' high parts summed with
    // TwoSum, all error terms summed in FP32, one renormalisation at the end.
    std::string dot(const std::vector<std::pair<std::string, std::string>>& t) {
        if (!ds_) {
            std::string acc = mul(t[0].first, t[0].second);
            for (size_t i = 1; i < t.size(); ++i) acc = fma(t[i].first, t[i].second, acc);
            return acc;
        }
        auto [s, err] = hl(ds_mul_raw(t[0].first, t[0].second));
        for (size_t i = 1; i < t.size(); ++i) {
            auto [p, e] = hl(ds_mul_raw(t[i].first, t[i].second));
            const std::string sn = f32op("add", s, p);
            const std::string v = f32op("sub", sn, s);
            const std::string r = f32op("add", f32op("sub", s, f32op("sub", sn, v)), f32op("sub", p, v));
            err = f32op("add", f32op("add", err, e), r);
            s = sn;
        }
        return s + "|" + err;
    }
    std::string add(const std::string& x, const std::string& y) {
        if (ds_) return ds_add(x, y);
        std::string d = A();
        I(fmt("add.rn.%s %s, %s, %s", ft_, d.c_str(), x.c_str(), y.c_str()));
        return d;
    }
    std::string sub(const std::string& x, const std::string& y) {
        if (ds_) return ds_add(x, neg(y));
        std::string d = A();
        I(fmt("sub.rn.%s %s, %s, %s", ft_, d.c_str(), x.c_str(), y.c_str()));
        return d;
    }
    // exact sign flip (FP64: on the integer high word, no FP64 instruction)
    std::string neg(const std::string& x) {
        if (ds_) {
            auto [h, l] = hl(x);
            return f32neg(h) + "|" + f32neg(l);
        }
        std::string d = A();
        if (f64_) {
            std::string t = R64(), u = R64();
            I(fmt("mov.b64 %s, %s", t.c_str(), x.c_str()));
            I(fmt("xor.b64 %s, %s, -9223372036854775808", u.c_str(), t.c_str()));
            I(fmt("mov.b64 %s, %s", d.c_str(), u.c_str()));
        } else {
            I(fmt("neg.f32 %s, %s", d.c_str(), x.c_str()));
        }
        return d;
    }
    std::string sel(const std::string& a, const std::string& b, const std::string& p) {  // p ? a : b
        if (ds_) {
            auto [ah, al] = hl(a);
            auto [bh, bl] = hl(b);
            std::string h = A(), l = A();
            I(fmt("selp.f32 %s, %s, %s, %s", h.c_str(), ah.c_str(), bh.c_str(), p.c_str()));
            I(fmt("selp.f32 %s, %s, %s, %s", l.c_str(), al.c_str(), bl.c_str(), p.c_str()));
            return h + "|" + l;
        }
        std::string d = A();
        I(fmt("selp.%s %s, %s, %s, %s", ft_, d.c_str(), a.c_str(), b.c_str(), p.c_str()));
        return d;
    }
    std::string f32const(float f) {
        uint32_t u;
        std::memcpy(&u, &f, 4);
        std::string d = A();
        I(fmt("mov.f32 %s, 0f%08X", d.c_str(), u));
        return d;
    }
    std::string cnst(double v) {
        auto it = consts_.find(v);
        if (it != consts_.end()) return it->second;
        std::string d;
        if (ds_) {
            const float h = static_cast<float>(v);
            const float l = static_cast<float>(v - static_cast<double>(h));
            d = f32const(h) + "|" + f32const(l);
        } else if (f64_) {
            d = A();
            uint64_t u;
            std::memcpy(&u, &v, 8);
            I(fmt("mov.f64 %s, 0d%016llX", d.c_str(), static_cast<unsigned long long>(u)));
        } else {
            d = f32const(static_cast<float>(v));
        }
        consts_[v] = d;
        return d;
    }
    // complex amplitude <-> shared memory (double-single: (re.h, re.l, im.h, im.l))
    Cx load_amp(const std::string& addr, uint32_t off) {
        if (ds_) {
            std::string r[4] = {A(), A(), A(), A()};
            I(fmt("ld.shared.v4.f32 {%s, %s, %s, %s}, [%s+%u]", r[0].c_str(), r[1].c_str(), r[2].c_str(),
                  r[3].c_str(), addr.c_str(), off));
            return {r[0] + "|" + r[1], r[2] + "|" + r[3]};
        }
        Cx c{A(), A()};
        I(fmt("ld.shared.v2.%s {%s, %s}, [%s+%u]", ft_, c.x.c_str(), c.y.c_str(), addr.c_str(), off));
        return c;
    }
    void store_amp(const std::string& addr, uint32_t off, const Cx& c, const std::string& pred = "") {
        const std::string g = pred.empty() ? "" : "@" + pred + " ";
        if (ds_) {
            auto [xh, xl] = hl(c.x);
            auto [yh, yl] = hl(c.y);
            I(fmt("%sst.shared.v4.f32 [%s+%u], {%s, %s, %s, %s}", g.c_str(), addr.c_str(), off, xh.c_str(),
                  xl.c_str(), yh.c_str(), yl.c_str()));
            return;
        }
        I(fmt("%sst.shared.v2.%s [%s+%u], {%s, %s}", g.c_str(), ft_, addr.c_str(), off, c.x.c_str(), c.y.c_str()));
    }
    // double-single <-> FP64 on the integer and FP32 pipes, no FP64
    // instruction (ds_from_double / ds_to_double of policy.cuh, step for step)
    std::string ds_from(const std::string& v) {
        std::string lw = R32(), hw = R32(), ah = R32(), f = R32(), sg = R32(), t = R32(), hb = R32();
        std::string ef = R32(), e2 = R32(), e3 = R32(), r23 = R32(), lb = R32(), lo = R32(), hz = R32(),
                    lz = R32();
        std::string tiny = P();
        std::string fl = A(), fe = A(), fd = A(), h = A(), l = A();
        I(fmt("mov.b64 {%s, %s}, %s", lw.c_str(), hw.c_str(), v.c_str()));
        I(fmt("and.b32 %s, %s, 0x7FFFFFFF", ah.c_str(), hw.c_str()));
        I(fmt("setp.lt.u32 %s, %s, 0x39800000", tiny.c_str(), ah.c_str()));  // |v| < 2^-103
        I(fmt("shf.l.clamp.b32 %s, %s, %s, 3", f.c_str(), lw.c_str(), hw.c_str()));
        I(fmt("and.b32 %s, %s, 0x80000000", sg.c_str(), hw.c_str()));
        I(fmt("xor.b32 %s, %s, 0x40000000", t.c_str(), f.c_str()));
        I(fmt("and.b32 %s, %s, 0x7FFFFFFF", t.c_str(), t.c_str()));
        I(fmt("or.b32 %s, %s, %s", hb.c_str(), t.c_str(), sg.c_str()));
        I(fmt("and.b32 %s, %s, 0x7F800000", ef.c_str(), f.c_str()));
        I(fmt("add.u32 %s, %s, 0x34800000", e2.c_str(), ef.c_str()));
        I(fmt("and.b32 %s, %s, 0x7F800000", e3.c_str(), e2.c_str()));
        I(fmt("bfe.u32 %s, %s, 6, 23", r23.c_str(), lw.c_str()));
        I(fmt("or.b32 %s, %s, %s", lb.c_str(), e3.c_str(), r23.c_str()));
        I(fmt("mov.b32 %s, %s", fl.c_str(), lb.c_str()));
        I(fmt("mov.b32 %s, %s", fe.c_str(), e3.c_str()));
        I(fmt("sub.rn.f32 %s, %s, %s", fd.c_str(), fl.c_str(), fe.c_str()));
        I(fmt("mov.b32 %s, %s", lo.c_str(), fd.c_str()));
        I(fmt("or.b32 %s, %s, %s", lo.c_str(), lo.c_str(), sg.c_str()));
        I(fmt("selp.b32 %s, %s, %s, %s", hz.c_str(), sg.c_str(), hb.c_str(), tiny.c_str()));
        I(fmt("selp.b32 %s, %s, %s, %s", lz.c_str(), sg.c_str(), lo.c_str(), tiny.c_str()));
        I(fmt("mov.b32 %s, %s", h.c_str(), hz.c_str()));
        I(fmt("mov.b32 %s, %s", l.c_str(), lz.c_str()));
        return h + "|" + l;
    }
    std::string ds_to(const std::string& vin) {
        const std::string v = ds_norm(vin);
        auto [h, l] = hl(v);
        std::string H = R32(), Lb = R32(), sh = R32(), eh = R32(), el = R32(), mh = R32(), ml = R32(), x = R32(),
                    d = R32(), z = R32(), ex = R32(), hi = R32(), lo = R32(), hw = R32(), hw2 = R32(), lw2 = R32();
        std::string MH = R64(), ML = R64(), MLs = R64(), Ms = R64(), Ma = R64(), M = R64(), Mn = R64(), mant = R64();
        std::string pel = P(), pneg = P(), pz = P();
        std::string out = D();
        I(fmt("mov.b32 %s, %s", H.c_str(), h.c_str()));
        I(fmt("mov.b32 %s, %s", Lb.c_str(), l.c_str()));
        I(fmt("and.b32 %s, %s, 0x80000000", sh.c_str(), H.c_str()));
        I(fmt("bfe.u32 %s, %s, 23, 8", eh.c_str(), H.c_str()));
        I(fmt("bfe.u32 %s, %s, 23, 8", el.c_str(), Lb.c_str()));
        I(fmt("and.b32 %s, %s, 0x007FFFFF", mh.c_str(), H.c_str()));
        I(fmt("or.b32 %s, %s, 0x00800000", mh.c_str(), mh.c_str()));
        I(fmt("and.b32 %s, %s, 0x007FFFFF", ml.c_str(), Lb.c_str()));
        I(fmt("or.b32 %s, %s, 0x00800000", ml.c_str(), ml.c_str()));
        I(fmt("xor.b32 %s, %s, %s", x.c_str(), H.c_str(), Lb.c_str()));
        I(fmt("setp.lt.s32 %s, %s, 0", pneg.c_str(), x.c_str()));  // opposite signs
        I(fmt("setp.eq.u32 %s, %s, 0", pel.c_str(), el.c_str()));
        I(fmt("sub.u32 %s, %s, %s", d.c_str(), eh.c_str(), el.c_str()));
        I(fmt("selp.b32 %s, 64, %s, %s", d.c_str(), d.c_str(), pel.c_str()));
        I(fmt("cvt.u64.u32 %s, %s", MH.c_str(), mh.c_str()));
        I(fmt("shl.b64 %s, %s, 39", MH.c_str(), MH.c_str()));
        I(fmt("cvt.u64.u32 %s, %s", ML.c_str(), ml.c_str()));
        I(fmt("shl.b64 %s, %s, 39", ML.c_str(), ML.c_str()));
        I(fmt("shr.b64 %s, %s, %s", MLs.c_str(), ML.c_str(), d.c_str()));
        I(fmt("sub.s64 %s, %s, %s", Ms.c_str(), MH.c_str(), MLs.c_str()));
        I(fmt("add.s64 %s, %s, %s", Ma.c_str(), MH.c_str(), MLs.c_str()));
        I(fmt("selp.b64 %s, %s, %s, %s", M.c_str(), Ms.c_str(), Ma.c_str(), pneg.c_str()));
        I(fmt("clz.b64 %s, %s", z.c_str(), M.c_str()));
        I(fmt("shl.b64 %s, %s, %s", Mn.c_str(), M.c_str(), z.c_str()));
        I(fmt("shr.b64 %s, %s, 11", mant.c_str(), Mn.c_str()));
        I(fmt("mov.b64 {%s, %s}, %s", lo.c_str(), hi.c_str(), mant.c_str()));
        I(fmt("sub.u32 %s, %s, %s", ex.c_str(), eh.c_str(), z.c_str()));
        I(fmt("add.u32 %s, %s, 896", ex.c_str(), ex.c_str()));
        I(fmt("shl.b32 %s, %s, 20", ex.c_str(), ex.c_str()));
        I(fmt("add.u32 %s, %s, %s", hw.c_str(), ex.c_str(), hi.c_str()));
        I(fmt("or.b32 %s, %s, %s", hw.c_str(), hw.c_str(), sh.c_str()));
        // h zero or below the FP32 normal range, or a cancelled pair: zero
        I(fmt("setp.eq.u32 %s, %s, 0", pz.c_str(), eh.c_str()));
        I(fmt("setp.eq.or.u32 %s, %s, 64, %s", pz.c_str(), z.c_str(), pz.c_str()));
        I(fmt("selp.b32 %s, %s, %s, %s", hw2.c_str(), sh.c_str(), hw.c_str(), pz.c_str()));
        I(fmt("selp.b32 %s, 0, %s, %s", lw2.c_str(), lo.c_str(), pz.c_str()));
        I(fmt("mov.b64 %s, {%s, %s}", out.c_str(), lw2.c_str(), hw2.c_str()));
        return out;
    }
    // coefficients off .. off+cnt-1 of the tile's pool (widest aligned loads)
    std::vector<std::string> coefs(uint32_t off, int cnt) {
        if (pc_) return pcoefs(off, cnt);
        std::vector<std::string> c;
        uint32_t i = off;
        const uint32_t end = off + cnt;
        while (i < end) {
            if (ds_) {  // (high, low) float pairs, two per 16-byte load
                if (i % 2 == 0 && i + 2 <= end) {
                    std::string r[4] = {A(), A(), A(), A()};
                    I(fmt("ld.global.nc.v4.f32 {%s, %s, %s, %s}, [%s+%u]", r[0].c_str(), r[1].c_str(),
                          r[2].c_str(), r[3].c_str(), coefp_.c_str(), i * cb_));
                    c.push_back(r[0] + "|" + r[1]);
                    c.push_back(r[2] + "|" + r[3]);
                    i += 2;
                } else {
                    std::string h = A(), l = A();
                    I(fmt("ld.global.nc.v2.f32 {%s, %s}, [%s+%u]", h.c_str(), l.c_str(), coefp_.c_str(), i * cb_));
                    c.push_back(h + "|" + l);
                    ++i;
                }
                continue;
            }
            int vec = 1;
            if (!f64_ && i % 4 == 0 && i + 4 <= end) vec = 4;
            else if (i % 2 == 0 && i + 2 <= end) vec = 2;
            std::string r[4];
            for (int k = 0; k < vec; ++k) r[k] = A();
            if (vec == 4)
                I(fmt("ld.global.nc.v4.f32 {%s, %s, %s, %s}, [%s+%u]", r[0].c_str(), r[1].c_str(), r[2].c_str(),
                      r[3].c_str(), coefp_.c_str(), i * cb_));
            else if (vec == 2)
                I(fmt("ld.global.nc.v2.%s {%s, %s}, [%s+%u]", ft_, r[0].c_str(), r[1].c_str(), coefp_.c_str(),
                      i * cb_));
            else
                I(fmt("ld.global.nc.%s %s, [%s+%u]", ft_, r[0].c_str(), coefp_.c_str(), i * cb_));
            for (int k = 0; k < vec; ++k) c.push_back(r[k]);
            i += vec;
        }
        return c;
    }

    // Coefficients from the pass's parameter block p_cblob (pool entries
    // cmin_ .. cmax_ in the arithmetic's format, warp-uniform constant
    // memory), one scalar load each, so each can become a constant operand.
    std::vector<std::string> pcoefs(uint32_t off, int cnt) {
        std::vector<std::string> c;
        for (uint32_t i = off; i < off + static_cast<uint32_t>(cnt); ++i) {
            const uint32_t rel = i - cmin_;
            if (ds_) {
                std::string h = A(), l = A();
                I(fmt("ld.param.f32 %s, [p_cblob+%u]", h.c_str(), rel * cb_));
                I(fmt("ld.param.f32 %s, [p_cblob+%u]", l.c_str(), rel * cb_ + 4));
                c.push_back(h + "|" + l);
            } else {
                std::string r = A();
                I(fmt("ld.param.%s %s, [p_cblob+%u]", ft_, r.c_str(), rel * cb_));
                c.push_back(r);
            }
        }
        return c;
    }

    // u64 register = OR over the set bits i of `r32` (bits 0..nbits-1) of val[i]
    std::string deposit64(const std::string& r32, int nbits, const std::vector<uint64_t>& val) {
        std::string acc = R64();
        I(fmt("mov.u64 %s, 0", acc.c_str()));
        for (int i = 0; i < nbits; ++i) {
            if (val[i] == 0) continue;
            std::string t = R32(), p = P(), v = R64(), n = R64();
            I(fmt("and.b32 %s, %s, %u", t.c_str(), r32.c_str(), 1u << i));
            I(fmt("setp.ne.u32 %s, %s, 0", p.c_str(), t.c_str()));
            I(fmt("selp.b64 %s, %llu, 0, %s", v.c_str(), static_cast<unsigned long long>(val[i]), p.c_str()));
            I(fmt("or.b64 %s, %s, %s", n.c_str(), acc.c_str(), v.c_str()));
            acc = n;
        }
        return acc;
    }
    // u32 register = sum over the set bits i of `r32` of val[i]
    std::string sum32(const std::string& r32, int nbits, const std::vector<uint32_t>& val) {
        std::string acc = R32();
        I(fmt("mov.u32 %s, 0", acc.c_str()));
        for (int i = 0; i < nbits; ++i) {
            if (val[i] == 0) continue;
            std::string t = R32(), n = R32();
            I(fmt("bfe.u32 %s, %s, %d, 1", t.c_str(), r32.c_str(), i));
            I(fmt("mad.lo.u32 %s, %s, %u, %s", n.c_str(), t.c_str(), val[i], acc.c_str()));
            acc = n;
        }
        return acc;
    }

    // ---------------------------------------------------------------- kernel
    void prologue() {
        tid_ = R32();
        I(fmt("mov.u32 %s, %%tid.x", tid_.c_str()));
        std::string bid = R32(), nbid = R32();
        I(fmt("mov.u32 %s, %%ctaid.x", bid.c_str()));
        I(fmt("mov.u32 %s, %%nctaid.x", nbid.c_str()));
        bid64_ = R64();
        nbid64_ = R64();
        I(fmt("cvt.u64.u32 %s, %s", bid64_.c_str(), bid.c_str()));
        I(fmt("cvt.u64.u32 %s, %s", nbid64_.c_str(), nbid.c_str()));
        const char* pn[2] = {"p_psi", "p_lam"};
        for (int s = 0; s < NS_; ++s) {
            std::string g = R64();
            stg_[s] = R64();
            I(fmt("ld.param.u64 %s, [%s]", g.c_str(), pn[s]));
            I(fmt("cvta.to.global.u64 %s, %s", stg_[s].c_str(), g.c_str()));
        }
        ntiles_ = R64();
        I(fmt("ld.param.u64 %s, [p_ntiles]", ntiles_.c_str()));
        std::string cg = R64();
        coef0_ = R64();
        I(fmt("ld.param.u64 %s, [p_coef]", cg.c_str()));
        I(fmt("cvta.to.global.u64 %s, %s", coef0_.c_str(), cg.c_str()));
        std::string cs = R64();
        cstrideB_ = R64();
        I(fmt("ld.param.u64 %s, [p_cstride]", cs.c_str()));
        I(fmt("mul.lo.u64 %s, %s, %d", cstrideB_.c_str(), cs.c_str(), cb_));
        ishift_ = R32();
        I(fmt("ld.param.u32 %s, [p_ishift]", ishift_.c_str()));
        if (NS_ == 1) {
            std::string ag = R64();
            active_ = R64();
            hasact_ = P();
            I(fmt("ld.param.u64 %s, [p_active]", ag.c_str()));
            I(fmt("setp.ne.u64 %s, %s, 0", hasact_.c_str(), ag.c_str()));
            I(fmt("cvta.to.global.u64 %s, %s", active_.c_str(), ag.c_str()));
        }
        smb_ = R32();
        I(fmt("mov.u32 %s, qsv_dsm", smb_.c_str()));
        std::string sg = R64();
        status_ = R64();
        I(fmt("ld.param.u64 %s, [p_status]", sg.c_str()));
        I(fmt("cvta.to.global.u64 %s, %s", status_.c_str(), sg.c_str()));
        waitns_ = R64();
        I(fmt("ld.param.u64 %s, [p_wait_ns]", waitns_.c_str()));
        extra_ = R32();
        I(fmt("ld.param.u32 %s, [p_extra_tx]", extra_.c_str()));
        if (bc_) {
            // bounds of the checked accesses: the dynamic shared memory, and
            // each state (ntiles tiles of 2^T amplitudes)
            smend_ = R32();
            Iraw(fmt("add.u32 %s, %s, %u", smend_.c_str(), smb_.c_str(), mbar_off() + 8u * sh_.nb));
            std::string nb = R64();
            Iraw(fmt("shl.b64 %s, %s, %d", nb.c_str(), ntiles_.c_str(), T_));
            std::string bytes = R64();
            Iraw(fmt("mul.lo.u64 %s, %s, %d", bytes.c_str(), nb.c_str(), es_));
            for (int st = 0; st < NS_; ++st) {
                gend_[st] = R64();
                Iraw(fmt("add.s64 %s, %s, %s", gend_[st].c_str(), stg_[st].c_str(), bytes.c_str()));
            }
        }
        // the thread's share of a tile: global byte offset and byte offset in
        // the tile layout; both are sums over the set bits of tid
        std::vector<uint64_t> gv(T_ - R_);
        std::vector<uint32_t> sv(T_ - R_);
        for (int i = 0; i < T_ - R_; ++i) {
            gv[i] = (1ULL << pd_.tq[i]) * es_;
            sv[i] = tile_weight(i, padu_) * es_;
        }
        gtidB_ = deposit64(tid_, T_ - R_, gv);
        stidB_ = sum32(tid_, T_ - R_, sv);
        std::string warp = R32();
        lane_ = R32();
        I(fmt("and.b32 %s, %s, 31", lane_.c_str(), tid_.c_str()));
        I(fmt("shr.u32 %s, %s, 5", warp.c_str(), tid_.c_str()));
        // bulk copies: thread r * 2^(L - R) moves run r of a tile (runs spread
        // over the warps, one per issuing thread and state); run r is global
        // byte offset grun(r) from the tile base and tile-layout offset
        // srun(r) in the slot, both sums over r's bits
        {
            const int sh = TILE_RUN_BITS - R_;  // log2(threads per run)
            iss_ = P();
            std::string low = R32(), run = R32();
            I(fmt("and.b32 %s, %s, %d", low.c_str(), tid_.c_str(), (1 << sh) - 1));
            I(fmt("setp.eq.u32 %s, %s, 0", iss_.c_str(), low.c_str()));
            I(fmt("shr.u32 %s, %s, %d", run.c_str(), tid_.c_str(), sh));
            std::vector<uint64_t> lg(H_);
            std::vector<uint32_t> ls(H_);
            for (int i = 0; i < H_; ++i) {
                lg[i] = grun(1u << i);
                ls[i] = srun(1u << i);
            }
            runG_ = deposit64(run, H_, lg);
            runS_ = sum32(run, H_, ls);
            runb_ = R32();
            I(fmt("mov.u32 %s, %u", runb_.c_str(), runB_));
            txb_ = R32();
            I(fmt("add.u32 %s, %s, %u", txb_.c_str(), extra_.c_str(), static_cast<uint32_t>(NS_) * (es_ << T_)));
        }
        // one mbarrier per tile slot, after the slots and the probe sums; thread
        // 0 registers each slot's expected bytes for its first phase (and for
        // every later phase right after the previous one completes), before
        // any copy of that phase is issued
        mbarB_ = R32();
        I(fmt("add.u32 %s, %s, %u", mbarB_.c_str(), smb_.c_str(), mbar_off()));
        t0_ = P();
        I(fmt("setp.eq.u32 %s, %s, 0", t0_.c_str(), tid_.c_str()));
        {
            const std::string lni = L();
            std::string pn = P();
            I(fmt("not.pred %s, %s", pn.c_str(), t0_.c_str()));
            I(fmt("@%s bra %s", pn.c_str(), lni.c_str()));
            for (int sl = 0; sl < sh_.nb; ++sl)
                I(fmt("mbarrier.init.shared::cta.b64 [%s+%d], 1", mbarB_.c_str(), 8 * sl));
            I("fence.mbarrier_init.release.cluster");
            for (int sl = 0; sl < sh_.nb; ++sl)
                I(fmt("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%s+%d], %s", mbarB_.c_str(), 8 * sl,
                      txb_.c_str()));
            I("fence.proxy.async.shared::cta");
            lab(lni);
        }
        if (np_ > 0) {
            paccB_ = R32();
            I(fmt("add.u32 %s, %s, %u", paccB_.c_str(), smb_.c_str(), slotB_ * sh_.nb));
            paccW_ = R32();
            I(fmt("mad.lo.u32 %s, %s, %d, %s", paccW_.c_str(), warp.c_str(), np_ * 8, paccB_.c_str()));
            std::string pt = R64();
            I(fmt("ld.param.u32 %s, [p_per_tile]", (perTile_ = R32()).c_str()));
            I(fmt("ld.param.u64 %s, [p_partial]", pt.c_str()));
            partial_ = R64();
            I(fmt("cvta.to.global.u64 %s, %s", partial_.c_str(), pt.c_str()));
            // zero the per-warp probe sums
            const int tot = NW_ * np_;
            for (int i0 = 0; i0 < tot; i0 += NT_) {
                std::string idx = R32(), p = P(), ad = R32();
                I(fmt("add.u32 %s, %s, %d", idx.c_str(), tid_.c_str(), i0));
                I(fmt("setp.lt.u32 %s, %s, %d", p.c_str(), idx.c_str(), tot));
                I(fmt("mad.lo.u32 %s, %s, 8, %s", ad.c_str(), idx.c_str(), paccB_.c_str()));
                I(fmt("@%s st.shared.u64 [%s], 0", p.c_str(), ad.c_str()));
            }
        }
        I("bar.sync 0");
    }

    // element index of the first amplitude of tile b (tile_base of device.cuh)
    std::string tile_base(const std::string& b) {
        std::string base = R64();
        I(fmt("shl.b64 %s, %s, %d", base.c_str(), b.c_str(), pd_.L));
        for (int k = 0; k < pd_.H; ++k) {
            const int p = pd_.tq[pd_.L + k];
            std::string hi = R64(), hi2 = R64(), lo = R64(), n = R64();
            I(fmt("shr.u64 %s, %s, %d", hi.c_str(), base.c_str(), p));
            I(fmt("shl.b64 %s, %s, %d", hi2.c_str(), hi.c_str(), p + 1));
            I(fmt("and.b64 %s, %s, %llu", lo.c_str(), base.c_str(), static_cast<unsigned long long>((1ULL << p) - 1)));
            I(fmt("or.b64 %s, %s, %s", n.c_str(), hi2.c_str(), lo.c_str()));
            base = n;
        }
        return base;
    }

    uint64_t gk(int k) const {  // global byte offset of element k * NT of a tile
        const uint32_t s = static_cast<uint32_t>(k * NT_);
        uint64_t g = 0;
        for (int i = 0; i < T_; ++i)
            if ((s >> i) & 1) g |= 1ULL << pd_.tq[i];
        return g * es_;
    }
    // tile-layout byte offset of element k * NT of a tile
    uint32_t sk(int k) const { return tile_off(static_cast<uint32_t>(k * NT_), padu_) * es_; }
    // global byte offset of run r of a tile from the tile's first amplitude
    uint64_t grun(uint32_t r) const {
        uint64_t g = 0;
        for (int k = 0; k < H_; ++k)
            if ((r >> k) & 1) g |= 1ULL << pd_.tq[TILE_RUN_BITS + k];
        return g * es_;
    }
    // tile-layout byte offset of run r in a slot
    uint32_t srun(uint32_t r) const { return tile_off(r << TILE_RUN_BITS, padu_) * es_; }
    // shared byte offset of the mbarriers: after the slots and the probe sums
    uint32_t mbar_off() const { return slotB_ * sh_.nb + static_cast<uint32_t>(NW_ * np_ * 8); }
    std::string gaddr_off(const std::string& gp, uint64_t off) {
        if (off < (1ULL << 31)) return gp + "+" + std::to_string(off);
        std::string a = R64();
        I(fmt("add.s64 %s, %s, %llu", a.c_str(), gp.c_str(), static_cast<unsigned long long>(off)));
        return a;
    }

    // per-thread global pointer of state s for tile base `base` (element index)
    std::string thread_gptr(int s, const std::string& base) {
        std::string bb = R64(), t = R64(), g = R64();
        I(fmt("mul.lo.u64 %s, %s, %d", bb.c_str(), base.c_str(), es_));
        I(fmt("add.s64 %s, %s, %s", t.c_str(), bb.c_str(), gtidB_.c_str()));
        I(fmt("add.s64 %s, %s, %s", g.c_str(), t.c_str(), stg_[s].c_str()));
        return g;
    }
    std::string gaddr(const std::string& gp, int k) {
        const uint64_t off = gk(k);
        if (off < (1ULL << 31)) return gp + "+" + std::to_string(off);
        std::string a = R64();
        I(fmt("add.s64 %s, %s, %llu", a.c_str(), gp.c_str(), static_cast<unsigned long long>(off)));
        return a;
    }

    // Bulk (TMA) copies of the tile at element `base` into the slot at shared
    // address `sbase`, completing on the mbarrier at `mbar` (whose expected
    // bytes are already registered): each issuing thread copies its run of
    // every state, after its own bulk stores of the slot's previous tile have
    // read their data.
    void prefetch(const std::string& base, const std::string& sbase, const std::string& mbar) {
        const std::string lskip = L();
        std::string ni = P();
        I(fmt("not.pred %s, %s", ni.c_str(), iss_.c_str()));
        I(fmt("@%s bra %s", ni.c_str(), lskip.c_str()));
        if (bulk_out_) I("cp.async.bulk.wait_group.read 0");
        std::string bb = R64(), gl = R64(), dl = R32();
        I(fmt("mul.lo.u64 %s, %s, %d", bb.c_str(), base.c_str(), es_));
        I(fmt("add.s64 %s, %s, %s", gl.c_str(), bb.c_str(), runG_.c_str()));
        I(fmt("add.u32 %s, %s, %s", dl.c_str(), sbase.c_str(), runS_.c_str()));
        for (int st = 0; st < NS_; ++st) {
            std::string g = R64();
            I(fmt("add.s64 %s, %s, %s", g.c_str(), gl.c_str(), stg_[st].c_str()));
            I(fmt("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%s+%u], [%s], %s, [%s]",
                  dl.c_str(), st * tileB_, g.c_str(), runb_.c_str(), mbar.c_str()));
        }
        lab(lskip);
    }

    // Bulk (TMA) stores of the slot at `sbase` to the tile at element `base`
    // (each issuing thread its run of every state), one bulk group per thread.
    void store_tile(const std::string& base, const std::string& sbase) {
        const std::string lskip = L();
        std::string ni = P();
        I(fmt("not.pred %s, %s", ni.c_str(), iss_.c_str()));
        I(fmt("@%s bra %s", ni.c_str(), lskip.c_str()));
        std::string bb = R64(), gl = R64(), dl = R32();
        I(fmt("mul.lo.u64 %s, %s, %d", bb.c_str(), base.c_str(), es_));
        I(fmt("add.s64 %s, %s, %s", gl.c_str(), bb.c_str(), runG_.c_str()));
        I(fmt("add.u32 %s, %s, %s", dl.c_str(), sbase.c_str(), runS_.c_str()));
        for (int st = 0; st < NS_; ++st) {
            std::string g = R64();
            I(fmt("add.s64 %s, %s, %s", g.c_str(), gl.c_str(), stg_[st].c_str()));
            I(fmt("cp.async.bulk.global.shared::cta.bulk_group [%s], [%s+%u], %s", g.c_str(), dl.c_str(),
                  st * tileB_, runb_.c_str()));
        }
        I("cp.async.bulk.commit_group");
        lab(lskip);
    }

    // Bounded wait for phase `par` of the mbarrier at `mbar`.  Returns a
    // predicate that is true when the wait gave up: p_wait_ns nanoseconds of
    // %globaltimer, or 2^26 polls, passed first.
    std::string wait_mbar(const std::string& mbar, const std::string& par) {
        const std::string ldone = L(), lloop = L();
        std::string ok = P(), to = P(), q = P(), q2 = P();
        I(fmt("setp.ne.u32 %s, %s, %s", to.c_str(), tid_.c_str(), tid_.c_str()));  // false
        I(fmt("mbarrier.try_wait.parity.shared::cta.b64 %s, [%s], %s", ok.c_str(), mbar.c_str(), par.c_str()));
        I(fmt("@%s bra %s", ok.c_str(), ldone.c_str()));
        std::string t0 = R64(), t1 = R64(), dt = R64(), cnt = R32();
        I(fmt("mov.u64 %s, %%globaltimer", t0.c_str()));
        I(fmt("mov.u32 %s, 0", cnt.c_str()));
        lab(lloop);
        I(fmt("mbarrier.try_wait.parity.shared::cta.b64 %s, [%s], %s", ok.c_str(), mbar.c_str(), par.c_str()));
        I(fmt("@%s bra %s", ok.c_str(), ldone.c_str()));
        I(fmt("add.u32 %s, %s, 1", cnt.c_str(), cnt.c_str()));
        I(fmt("mov.u64 %s, %%globaltimer", t1.c_str()));
        I(fmt("sub.u64 %s, %s, %s", dt.c_str(), t1.c_str(), t0.c_str()));
        I(fmt("setp.lt.u64 %s, %s, %s", q.c_str(), dt.c_str(), waitns_.c_str()));
        I(fmt("setp.lt.and.u32 %s, %s, %u, %s", q2.c_str(), cnt.c_str(), 1u << 26, q.c_str()));
        I(fmt("@%s bra %s", q2.c_str(), lloop.c_str()));
        I(fmt("setp.eq.u32 %s, %s, %s", to.c_str(), tid_.c_str(), tid_.c_str()));  // true
        lab(ldone);
        return to;
    }

    void tile_loop() {
        std::string b = R64();
        I(fmt("mov.u64 %s, %s", b.c_str(), bid64_.c_str()));
        const std::string lend = L(), lloop = L(), lfail = L();
        std::string p0 = P();
        I(fmt("setp.ge.u64 %s, %s, %s", p0.c_str(), b.c_str(), ntiles_.c_str()));
        I(fmt("@%s bra %s", p0.c_str(), lend.c_str()));
        // loop-carried: slot byte offset, slot index, per-slot mbarrier parities
        std::string slot = R32(), sidx = R32(), phase = R32();
        I(fmt("mov.u32 %s, 0", slot.c_str()));
        I(fmt("mov.u32 %s, 0", sidx.c_str()));
        I(fmt("mov.u32 %s, 0", phase.c_str()));
        std::string cmbar = R32(), cpar = R32(), omb = R32(), opar = R32(), nextp = P();
        if (sh_.nb == 2) {
            std::string base0 = tile_base(b);
            prefetch(base0, smb_, mbarB_);
        }
        lab(lloop);
        // loop-carried registers are re-assigned at the end of the body
        std::string base = tile_base(b);
        std::string item = R64(), coff = R64();
        I(fmt("shr.u64 %s, %s, %s", item.c_str(), b.c_str(), ishift_.c_str()));
        I(fmt("mul.lo.u64 %s, %s, %s", coff.c_str(), item.c_str(), cstrideB_.c_str()));
        coefp_ = R64();
        I(fmt("add.s64 %s, %s, %s", coefp_.c_str(), coef0_.c_str(), coff.c_str()));
        std::string sbase = R32();
        I(fmt("add.u32 %s, %s, %s", sbase.c_str(), smb_.c_str(), slot.c_str()));
        I(fmt("mad.lo.u32 %s, %s, 8, %s", cmbar.c_str(), sidx.c_str(), mbarB_.c_str()));
        I(fmt("bfe.u32 %s, %s, %s, 1", cpar.c_str(), phase.c_str(), sidx.c_str()));
        // Two slots: the next tile goes into the other slot while this one is
        // computed.  With bulk stores (not double-single) its copies are
        // issued after the tile's first step, by when the stores of the
        // slot's previous tile have read it out; otherwise at once.
        // `nextp` (set where the copies are issued) tells the failure path
        // which waits have copies behind them.
        std::string bn = R64(), nsb = R32();
        I(fmt("setp.ne.u32 %s, %s, %s", nextp.c_str(), tid_.c_str(), tid_.c_str()));  // false
        auto next_prefetch = [&] {
            std::string pn = P(), nslot = R32(), osidx = R32();
            const std::string lno = L();
            I(fmt("add.s64 %s, %s, %s", bn.c_str(), b.c_str(), nbid64_.c_str()));
            I(fmt("setp.lt.u64 %s, %s, %s", nextp.c_str(), bn.c_str(), ntiles_.c_str()));
            I(fmt("xor.b32 %s, %s, 1", osidx.c_str(), sidx.c_str()));
            I(fmt("mad.lo.u32 %s, %s, 8, %s", omb.c_str(), osidx.c_str(), mbarB_.c_str()));
            I(fmt("bfe.u32 %s, %s, %s, 1", opar.c_str(), phase.c_str(), osidx.c_str()));
            I(fmt("not.pred %s, %s", pn.c_str(), nextp.c_str()));
            I(fmt("@%s bra %s", pn.c_str(), lno.c_str()));
            I(fmt("xor.b32 %s, %s, %u", nslot.c_str(), slot.c_str(), slotB_));
            I(fmt("add.u32 %s, %s, %s", nsb.c_str(), smb_.c_str(), nslot.c_str()));
            std::string nbase = tile_base(bn);
            prefetch(nbase, nsb, omb);
            lab(lno);
        };
        const bool late_next = sh_.nb == 2 && bulk_out_ && pd_.step_count > 0;
        if (sh_.nb == 1) prefetch(base, sbase, cmbar);
        else if (!late_next) next_prefetch();
        {
            const std::string to = wait_mbar(cmbar, cpar);
            std::string pf = P(), t = R32();
            I(fmt("bar.red.or.pred %s, 0, %s", pf.c_str(), to.c_str()));
            I(fmt("@%s bra %s", pf.c_str(), lfail.c_str()));
            I(fmt("add.u32 %s, %s, 1", t.c_str(), sidx.c_str()));  // 1 << sidx
            I(fmt("xor.b32 %s, %s, %s", phase.c_str(), phase.c_str(), t.c_str()));
            // every thread has seen this phase complete: register the bytes of
            // the slot's next phase before any of its copies is issued
            I(fmt("@%s mbarrier.arrive.expect_tx.shared::cta.b64 _, [%s], %s", t0_.c_str(), cmbar.c_str(),
                  txb_.c_str()));
        }
        note("tile staged: conversions");
        // the thread's tile-layout base in this slot
        std::string tbase = R32();
        I(fmt("add.u32 %s, %s, %s", tbase.c_str(), stidB_.c_str(), sbase.c_str()));
        if (ds_ && !in_pair_) {
            for (int k = 0; k < PER_; ++k) {
                for (int st = 0; st < NS_; ++st) {
                    std::string re = D(), im = D();
                    I(fmt("ld.shared.v2.f64 {%s, %s}, [%s+%u]", re.c_str(), im.c_str(), tbase.c_str(),
                          st * tileB_ + sk(k)));
                    store_amp(tbase, st * tileB_ + sk(k), {ds_from(re), ds_from(im)});
                }
            }
            I("bar.sync 0");
        }

        for (int si = 0; si < pd_.step_count; ++si) {
            const StepDesc& sd = hp_.steps[pd_.step_begin + si];
            if (sd.type == STEP_SMEM) smem_step(sd, base, sbase);
            else round(sd, base, sbase);
            if (si == 0 && late_next) next_prefetch();
        }

        note("write-back");
        // write the tile back (one-state passes: only active items)
        const std::string lskip = L();
        if (NS_ == 1) {
            const std::string lst = L();
            std::string nact = P();
            I(fmt("not.pred %s, %s", nact.c_str(), hasact_.c_str()));
            I(fmt("@%s bra %s", nact.c_str(), lst.c_str()));
            std::string ap = R64(), av = H16(), pz = P();
            I(fmt("add.s64 %s, %s, %s", ap.c_str(), active_.c_str(), item.c_str()));
            I(fmt("ld.global.u8 %s, [%s]", av.c_str(), ap.c_str()));
            I(fmt("setp.eq.u16 %s, %s, 0", pz.c_str(), av.c_str()));
            I(fmt("@%s bra %s", pz.c_str(), lskip.c_str()));
            lab(lst);
        }
        if (out_pair_) {
            // float pairs for the next pass: renormalised (TwoSum) once here,
            // so |low| stays within half an ulp of high from pass to pass
            for (int k = 0; k < PER_; ++k)
                for (int st = 0; st < NS_; ++st) {
                    const Cx c = load_amp(tbase, st * tileB_ + sk(k));
                    store_amp(tbase, st * tileB_ + sk(k), {ds_norm(c.x), ds_norm(c.y)});
                }
        }
        if (ds_ && !out_pair_) {
            for (int st = 0; st < NS_; ++st) {
                std::string gp = thread_gptr(st, base);
                for (int k = 0; k < PER_; ++k) {
                    const std::string dst = gaddr(gp, k);
                    const Cx c = load_amp(tbase, st * tileB_ + sk(k));
                    const std::string re = ds_to(c.x), im = ds_to(c.y);
                    I(fmt("st.global.cs.v2.f64 [%s], {%s, %s}", dst.c_str(), re.c_str(), im.c_str()));
                }
            }
        } else {
            // the rounds' shared-memory writes, then bulk (TMA) stores of the runs
            I("fence.proxy.async.shared::cta");
            I("bar.sync 0");
            store_tile(base, sbase);
        }
        lab(lskip);
        I("bar.sync 0");
        if (np_ > 0) {
            // batched runs: this tile's probe sums, then zero them
            const std::string lnp = L();
            std::string pp = P(), pin = P();
            I(fmt("setp.eq.u32 %s, %s, 0", pp.c_str(), perTile_.c_str()));
            I(fmt("@%s bra %s", pp.c_str(), lnp.c_str()));
            I(fmt("setp.lt.u32 %s, %s, %d", pin.c_str(), tid_.c_str(), np_));
            const std::string lno = L();
            std::string npin = P();
            I(fmt("not.pred %s, %s", npin.c_str(), pin.c_str()));
            I(fmt("@%s bra %s", npin.c_str(), lno.c_str()));
            std::string a0 = R32();
            I(fmt("mad.lo.u32 %s, %s, 8, %s", a0.c_str(), tid_.c_str(), paccB_.c_str()));
            std::string s = D();
            I(fmt("mov.f64 %s, 0d0000000000000000", s.c_str()));
            for (int w = 0; w < NW_; ++w) {
                std::string v = D(), n = D();
                I(fmt("ld.shared.f64 %s, [%s+%d]", v.c_str(), a0.c_str(), w * np_ * 8));
                I(fmt("add.rn.f64 %s, %s, %s", n.c_str(), s.c_str(), v.c_str()));
                I(fmt("st.shared.u64 [%s+%d], 0", a0.c_str(), w * np_ * 8));
                s = n;
            }
            std::string t64 = R64(), ix = R64(), ad = R64();
            I(fmt("cvt.u64.u32 %s, %s", t64.c_str(), tid_.c_str()));
            I(fmt("mad.lo.u64 %s, %s, %s, %s", ix.c_str(), t64.c_str(), ntiles_.c_str(), b.c_str()));
            I(fmt("mad.lo.u64 %s, %s, 8, %s", ad.c_str(), ix.c_str(), partial_.c_str()));
            I(fmt("st.global.f64 [%s], %s", ad.c_str(), s.c_str()));
            lab(lno);
            I("bar.sync 0");
            lab(lnp);
        }
        // next tile (PTX registers are not SSA: the loop variables are updated in place)
        I(fmt("add.s64 %s, %s, %s", b.c_str(), b.c_str(), nbid64_.c_str()));
        if (sh_.nb == 2) {
            I(fmt("xor.b32 %s, %s, %u", slot.c_str(), slot.c_str(), slotB_));
            I(fmt("xor.b32 %s, %s, 1", sidx.c_str(), sidx.c_str()));
        }
        std::string pc = P();
        I(fmt("setp.lt.u64 %s, %s, %s", pc.c_str(), b.c_str(), ntiles_.c_str()));
        I(fmt("@%s bra %s", pc.c_str(), lloop.c_str()));
        lab(lend);
        if (bulk_out_) I(fmt("@%s cp.async.bulk.wait_group 0", iss_.c_str()));  // the last tile's stores
        if (np_ > 0) {
            // single state: this CTA's per-probe totals
            const std::string lx = L();
            std::string pp = P(), pin = P();
            I(fmt("setp.ne.u32 %s, %s, 0", pp.c_str(), perTile_.c_str()));
            I(fmt("@%s bra %s", pp.c_str(), lx.c_str()));
            I("bar.sync 0");
            I(fmt("setp.ge.u32 %s, %s, %d", pin.c_str(), tid_.c_str(), np_));
            I(fmt("@%s bra %s", pin.c_str(), lx.c_str()));
            std::string a0 = R32();
            I(fmt("mad.lo.u32 %s, %s, 8, %s", a0.c_str(), tid_.c_str(), paccB_.c_str()));
            std::string s = D();
            I(fmt("mov.f64 %s, 0d0000000000000000", s.c_str()));
            for (int w = 0; w < NW_; ++w) {
                std::string v = D(), n = D();
                I(fmt("ld.shared.f64 %s, [%s+%d]", v.c_str(), a0.c_str(), w * np_ * 8));
                I(fmt("add.rn.f64 %s, %s, %s", n.c_str(), s.c_str(), v.c_str()));
                s = n;
            }
            std::string t64 = R64(), ix = R64(), ad = R64();
            I(fmt("cvt.u64.u32 %s, %s", t64.c_str(), tid_.c_str()));
            I(fmt("mad.lo.u64 %s, %s, %s, %s", ix.c_str(), t64.c_str(), nbid64_.c_str(), bid64_.c_str()));
            I(fmt("mad.lo.u64 %s, %s, 8, %s", ad.c_str(), ix.c_str(), partial_.c_str()));
            I(fmt("st.global.f64 [%s], %s", ad.c_str(), s.c_str()));
            lab(lx);
        }
        I("ret");
        // A tile's copies did not complete in time (every thread of the CTA
        // agreed through bar.red): record QFVM_ERR_TIMEOUT, wait (bounded)
        // for the copies still in flight, let warp 0's bulk stores finish
        // reading, and leave without another barrier.
        lab(lfail);
        {
            std::string p0t = P();
            I(fmt("setp.eq.u32 %s, %s, 0", p0t.c_str(), tid_.c_str()));
            std::string old = R32();  // the first error recorded stays
            I(fmt("@%s atom.global.cas.b32 %s, [%s], 0, %d", p0t.c_str(), old.c_str(), status_.c_str(),
                  static_cast<int>(QFVM_ERR_TIMEOUT)));
            wait_mbar(cmbar, cpar);
            if (sh_.nb == 2) {
                const std::string lno = L();
                std::string pn = P();
                I(fmt("not.pred %s, %s", pn.c_str(), nextp.c_str()));
                I(fmt("@%s bra %s", pn.c_str(), lno.c_str()));
                wait_mbar(omb, opar);
                lab(lno);
            }
            if (bulk_out_) I(fmt("@%s cp.async.bulk.wait_group 0", iss_.c_str()));
            I("ret");
        }
    }

    // ---------------------------------------------------------------- rounds
    std::string ctl_pred(const KOp& o, const std::string& gthr) {
        std::string t = R64(), p = P();
        I(fmt("and.b64 %s, %s, %llu", t.c_str(), gthr.c_str(), static_cast<unsigned long long>(o.cthr)));
        I(fmt("setp.eq.u64 %s, %s, %llu", p.c_str(), t.c_str(), static_cast<unsigned long long>(o.cthr)));
        return p;
    }
    std::string par_pred(const KOp& o, const std::string& gthr) {
        std::string t = R64(), c = R32(), c1 = R32(), p = P();
        I(fmt("and.b64 %s, %s, %llu", t.c_str(), gthr.c_str(), static_cast<unsigned long long>(o.pthr)));
        I(fmt("popc.b64 %s, %s", c.c_str(), t.c_str()));
        I(fmt("and.b32 %s, %s, 1", c1.c_str(), c.c_str()));
        I(fmt("setp.ne.u32 %s, %s, 0", p.c_str(), c1.c_str()));
        return p;
    }

    Cx phase(const Cx& a, const std::string& dr, const std::string& di, const std::string& ndi) {
        // amp_phase: a * (dr + i di)
        return {dot({{dr, a.x}, {ndi, a.y}}), dot({{dr, a.y}, {di, a.x}})};
    }
    Cx special(const Cx& a, int sp) {  // amp_special: * -1, * i, * -i
        if (sp == SP_NEG1) return {neg(a.x), neg(a.y)};
        if (sp == SP_I) return {neg(a.y), a.x};
        return {a.y, neg(a.x)};
    }
    Cx special_value(int sp) {
        if (sp == SP_NEG1) return {cnst(-1.0), cnst(0.0)};
        if (sp == SP_I) return {cnst(0.0), cnst(1.0)};
        return {cnst(0.0), cnst(-1.0)};
    }
    Cx rot_q(const Cx& a, const std::string& s1, const std::string& s2) {  // a * i^q, q = s1 + 2 s2
        Cx t{sel(neg(a.y), a.x, s1), sel(a.x, a.y, s1)};
        return {sel(neg(t.x), t.x, s2), sel(neg(t.y), t.y, s2)};
    }

    std::vector<int> pairs(int t, uint32_t creg) const {
        std::vector<int> v;
        for (int j = 0; j < NA_; ++j)
            if (!((j >> t) & 1) && (static_cast<uint32_t>(j) & creg) == creg) v.push_back(j);
        return v;
    }

    // the two diagonal entries of a DIAG op (constants where the flags fix them)
    void diag_entries(const KOp& o, Cx* d0, Cx* d1) {
        std::vector<std::string> c;
        const bool need_load = !(o.flags & F_D0_ONE) || !(o.flags & F_D1_SPEC);
        if (need_load) c = coefs(o.coef, 4);
        *d0 = (o.flags & F_D0_ONE) ? Cx{cnst(1.0), cnst(0.0)} : Cx{c[0], c[1]};
        *d1 = (o.flags & F_D1_SPEC) ? special_value(o.special) : Cx{c[2], c[3]};
    }

    void op_diag(const KOp& o, const std::string& gthr, const std::string& ctl) {
        const bool tpar = (o.flags & F_TPAR) != 0;
        std::string pt = tpar ? par_pred(o, gthr) : "";
        if (o.flags & F_UNIFORM) {
            if (!tpar) {
                if (o.flags & F_D0_ONE) return;
                std::vector<std::string> c = coefs(o.coef, 2);
                phase_mul({c[0], c[1]}, ctl);
                return;
            }
            if ((o.flags & F_D0_ONE) && (o.flags & F_D1_SPEC)) {
                const int qa = o.special == SP_NEG1 ? 2 : (o.special == SP_I ? 1 : 3);
                std::string pa = pt;
                if (!ctl.empty()) {
                    pa = P();
                    I(fmt("and.pred %s, %s, %s", pa.c_str(), pt.c_str(), ctl.c_str()));
                }
                std::string v = R32(), nq = R32();
                I(fmt("selp.b32 %s, %d, 0, %s", v.c_str(), qa, pa.c_str()));
                if (q_.empty()) {
                    q_ = v;
                } else {
                    I(fmt("add.u32 %s, %s, %s", nq.c_str(), q_.c_str(), v.c_str()));
                    q_ = nq;
                }
                return;
            }
            Cx d0, d1;
            diag_entries(o, &d0, &d1);
            phase_mul({sel(d1.x, d0.x, pt), sel(d1.y, d0.y, pt)}, ctl);
            return;
        }
        auto old = A_;
        if (o.flags & F_ONEBIT) {
            const int t = o.t0;
            if (!tpar) {
                std::vector<std::string> c;
                if (!(o.flags & F_D0_ONE) || !(o.flags & F_D1_SPEC)) c = coefs(o.coef, 4);
                for (int j = 0; j < NA_; ++j) {
                    const int h = (j >> t) & 1;
                    for (int s = 0; s < NS_; ++s) {
                        if (h == 0) {
                            if (o.flags & F_D0_ONE) continue;
                            A_[s][j] = phase(A_[s][j], c[0], c[1], neg(c[1]));
                        } else if (o.flags & F_D1_SPEC) {
                            A_[s][j] = special(A_[s][j], o.special);
                        } else {
                            A_[s][j] = phase(A_[s][j], c[2], c[3], neg(c[3]));
                        }
                    }
                }
            } else {
                Cx d0, d1;
                diag_entries(o, &d0, &d1);
                Cx f[2] = {{sel(d1.x, d0.x, pt), sel(d1.y, d0.y, pt)}, {sel(d0.x, d1.x, pt), sel(d0.y, d1.y, pt)}};
                std::string nf[2] = {neg(f[0].y), neg(f[1].y)};
                for (int j = 0; j < NA_; ++j) {
                    const int h = (j >> t) & 1;
                    for (int s = 0; s < NS_; ++s) A_[s][j] = phase(A_[s][j], f[h].x, f[h].y, nf[h]);
                }
            }
        } else {
            // parity over register bits (and the thread's), register controls
            Cx d0, d1;
            std::vector<std::string> c = coefs(o.coef, 4);
            d0 = {c[0], c[1]};
            d1 = {c[2], c[3]};
            Cx f[2] = {d0, d1};
            if (tpar) {
                f[0] = {sel(d1.x, d0.x, pt), sel(d1.y, d0.y, pt)};
                f[1] = {sel(d0.x, d1.x, pt), sel(d0.y, d1.y, pt)};
            }
            std::string nf[2] = {neg(f[0].y), neg(f[1].y)};
            for (int j = 0; j < NA_; ++j) {
                if ((static_cast<uint32_t>(j) & o.creg) != o.creg) continue;
                const int par = __builtin_popcount(static_cast<uint32_t>(j) & o.preg) & 1;
                for (int s = 0; s < NS_; ++s) A_[s][j] = phase(A_[s][j], f[par].x, f[par].y, nf[par]);
            }
        }
        guard(old, ctl);
    }

    // merged register-round diagonal: entry j multiplies register j (exact
    // entries 1, -1, i, -i without arithmetic)
    void op_diagr(const KOp& o) {
        for (int j = 0; j < NA_; ++j) {
            const int code = diagr_code(o, j);
            if (code == DIAGR_ONE) continue;
            if (code != DIAGR_GENERAL) {
                const int sp = code == DIAGR_NEG1 ? SP_NEG1 : (code == DIAGR_I ? SP_I : SP_NEGI);
                for (int s = 0; s < NS_; ++s) A_[s][j] = special(A_[s][j], sp);
                continue;
            }
            // each entry's coefficients just before their use (a table of 2^R
            // entries loaded at once would hold 2^(R+1) registers)
            const std::vector<std::string> c = coefs(o.coef + 2 * j, 2);
            const std::string dr = c[0], di = c[1], ndi = neg(di);
            for (int s = 0; s < NS_; ++s) A_[s][j] = phase(A_[s][j], dr, di, ndi);
        }
    }

    // round phase *= f (only where ctl holds, when given)
    void phase_mul(const Cx& f, const std::string& ctl) {
        Cx n;
        if (!ph_on_) {
            n = f;
            if (!ctl.empty()) n = {sel(f.x, cnst(1.0), ctl), sel(f.y, cnst(0.0), ctl)};
        } else {
            n = phase(ph_, f.x, f.y, neg(f.y));
            if (!ctl.empty()) n = {sel(n.x, ph_.x, ctl), sel(n.y, ph_.y, ctl)};
        }
        ph_ = n;
        ph_on_ = true;
    }

    // thread-controlled op: keep the old values where the control is 0
    void guard(const std::vector<std::vector<Cx>>& old, const std::string& ctl) {
        if (ctl.empty()) return;
        for (int s = 0; s < NS_; ++s)
            for (int j = 0; j < NA_; ++j)
                if (!same(A_[s][j], old[s][j]))
                    A_[s][j] = {sel(A_[s][j].x, old[s][j].x, ctl), sel(A_[s][j].y, old[s][j].y, ctl)};
    }

    void op_gate(const KOp& o, const std::string& ctl) {
        auto old = A_;
        const int t = o.t0;
        switch (o.kind) {
            case K_X:
                for (int j : pairs(t, o.creg))
                    for (int s = 0; s < NS_; ++s) std::swap(A_[s][j], A_[s][j | (1 << t)]);
                break;
            case K_Y:
                for (int j : pairs(t, o.creg))
                    for (int s = 0; s < NS_; ++s) {
                        const Cx a = A_[s][j], b = A_[s][j | (1 << t)];
                        A_[s][j] = {b.y, neg(b.x)};
                        A_[s][j | (1 << t)] = {neg(a.y), a.x};
                    }
                break;
            case K_HAD:
                for (int j : pairs(t, o.creg))
                    for (int s = 0; s < NS_; ++s) {
                        const Cx a = A_[s][j], b = A_[s][j | (1 << t)];
                        A_[s][j] = {add(a.x, b.x), add(a.y, b.y)};
                        A_[s][j | (1 << t)] = {sub(a.x, b.x), sub(a.y, b.y)};
                    }
                break;
            case K_REAL: {
                std::vector<std::string> m = coefs(o.coef, 4);
                if (!flip_[t].empty()) {  // X U X = [[m3, m2], [m1, m0]] where the thread's bit t is flipped
                    const std::string& p = flip_[t];
                    m = {sel(m[3], m[0], p), sel(m[2], m[1], p), sel(m[1], m[2], p), sel(m[0], m[3], p)};
                }
                for (int j : pairs(t, o.creg))
                    for (int s = 0; s < NS_; ++s) {
                        const Cx a = A_[s][j], b = A_[s][j | (1 << t)];
                        A_[s][j] = {dot({{m[0], a.x}, {m[1], b.x}}), dot({{m[0], a.y}, {m[1], b.y}})};
                        A_[s][j | (1 << t)] = {dot({{m[2], a.x}, {m[3], b.x}}), dot({{m[2], a.y}, {m[3], b.y}})};
                    }
                break;
            }
            case K_RX: {
                std::vector<std::string> m = coefs(o.coef, 2);
                const std::string c = m[0], sn = m[1], ns = neg(m[1]);
                for (int j : pairs(t, o.creg))
                    for (int s = 0; s < NS_; ++s) {
                        const Cx a = A_[s][j], b = A_[s][j | (1 << t)];
                        A_[s][j] = {dot({{c, a.x}, {sn, b.y}}), dot({{c, a.y}, {ns, b.x}})};
                        A_[s][j | (1 << t)] = {dot({{c, b.x}, {sn, a.y}}), dot({{c, b.y}, {ns, a.x}})};
                    }
                break;
            }
            case K_DENSE: {
                std::vector<std::string> m = coefs(o.coef, 8);
                if (!flip_[t].empty()) {  // X U X: (m00, m01, m10, m11) -> (m11, m10, m01, m00)
                    const std::string& p = flip_[t];
                    std::vector<std::string> f(8);
                    for (int e = 0; e < 4; ++e)
                        for (int c = 0; c < 2; ++c) f[2 * e + c] = sel(m[2 * (3 - e) + c], m[2 * e + c], p);
                    m = f;
                }
                std::string nmi[4];
                for (int i = 0; i < 4; ++i) nmi[i] = neg(m[2 * i + 1]);
                for (int j : pairs(t, o.creg))
                    for (int s = 0; s < NS_; ++s) {
                        const Cx a = A_[s][j], b = A_[s][j | (1 << t)];
                        A_[s][j] = {dot({{m[0], a.x}, {nmi[0], a.y}, {m[2], b.x}, {nmi[1], b.y}}),
                                    dot({{m[0], a.y}, {m[1], a.x}, {m[2], b.y}, {m[3], b.x}})};
                        A_[s][j | (1 << t)] = {dot({{m[4], a.x}, {nmi[2], a.y}, {m[6], b.x}, {nmi[3], b.y}}),
                                               dot({{m[4], a.y}, {m[5], a.x}, {m[6], b.y}, {m[7], b.x}})};
                    }
                break;
            }
            case K_SWAP: {
                const int lo = o.t0 < o.t1 ? o.t0 : o.t1, hi = o.t0 < o.t1 ? o.t1 : o.t0;
                std::swap(flip_[lo], flip_[hi]);
                for (int j = 0; j < NA_; ++j) {
                    if (j & ((1 << lo) | (1 << hi))) continue;
                    if ((static_cast<uint32_t>(j) & o.creg) != o.creg) continue;
                    for (int s = 0; s < NS_; ++s) std::swap(A_[s][j | (1 << lo)], A_[s][j | (1 << hi)]);
                }
                break;
            }
            default: break;
        }
        guard(old, ctl);
    }

    // Im<lam| Q |psi> share of the thread (probe_sum / reg_probe of
    // adjoint.cuh, the register terms summed as a balanced tree).  The
    // thread values of up to 8 probes wait in registers and are warp-summed
    // together (flush_probes).
    void op_probe(const KOp& o, const std::string& gthr, const std::string& ctl) {
        struct Term {
            std::string r;
            bool neg;
        };
        std::vector<Term> tr, ti;
        for (int j = 0; j < NA_; ++j) {
            if ((static_cast<uint32_t>(j) & o.creg) != o.creg) continue;
            const int jx = j ^ static_cast<int>(o.xreg);
            const bool ng = (__builtin_popcount(static_cast<uint32_t>(jx) & o.preg) & 1) != 0;
            const Cx l = A_[1][j], w = A_[0][jx];
            tr.push_back({fma(l.x, w.x, mul(l.y, w.y)), ng});
            ti.push_back({fma(l.x, w.y, neg(mul(l.y, w.x))), ng});
        }
        auto tree = [&](std::vector<Term> t) -> std::string {
            if (t.empty()) return cnst(0.0);
            while (t.size() > 1) {
                std::vector<Term> n;
                for (size_t i = 0; i + 1 < t.size(); i += 2) {
                    const Term& a = t[i];
                    const Term& b = t[i + 1];
                    if (a.neg == b.neg) n.push_back({add(a.r, b.r), a.neg});
                    else if (a.neg) n.push_back({sub(b.r, a.r), false});
                    else n.push_back({sub(a.r, b.r), false});
                }
                if (t.size() & 1) n.push_back(t.back());
                t.swap(n);
            }
            return t[0].neg ? neg(t[0].r) : t[0].r;
        };
        const std::string ar = tree(tr), ai = tree(ti);
        std::string v;
        switch (o.special & 3) {
            case 0: v = ai; break;
            case 1: v = ar; break;
            case 2: v = neg(ai); break;
            default: v = neg(ar); break;
        }
        if (o.flags & F_TPAR) {
            std::string pt = par_pred(o, gthr);
            v = sel(neg(v), v, pt);
        }
        if (!ctl.empty()) v = sel(v, cnst(0.0), ctl);
        if (ds_) v = ds_to(v);  // warp sums in FP64
        pending_.push_back({v, static_cast<int>(o.probe), o.coef});
        if (static_cast<int>(pending_.size()) == (f64_ ? 4 : 8)) flush_probes();
    }

    // Warp sums of the pending probes with one butterfly: at each of the
    // first log2(P) exchanges a lane keeps half of its values and sends the
    // other half, so P values cost about P shuffles instead of 5 P.  Lane L
    // ends with probe L >> (5 - log2 P); the first lane of each group adds
    // the warp total (times the generator scale) to this warp's slot.
    // probe-value arithmetic: the amplitude type, or FP64 for double-single
    std::string pzero() {
        if (!ds_) return cnst(0.0);
        std::string d = D();
        I(fmt("mov.f64 %s, 0d0000000000000000", d.c_str()));
        return d;
    }
    std::string psel(const std::string& a, const std::string& b, const std::string& p) {
        if (!ds_) return sel(a, b, p);
        std::string d = D();
        I(fmt("selp.f64 %s, %s, %s, %s", d.c_str(), a.c_str(), b.c_str(), p.c_str()));
        return d;
    }
    std::string padd(const std::string& a, const std::string& b) {
        if (!ds_) return add(a, b);
        std::string d = D();
        I(fmt("add.rn.f64 %s, %s, %s", d.c_str(), a.c_str(), b.c_str()));
        return d;
    }
    std::string pshfl(const std::string& v, int lanemask) {
        if (!ds_) return shfl(v, lanemask);
        std::string lo = R32(), hi = R32(), lo2 = R32(), hi2 = R32(), d = D();
        I(fmt("mov.b64 {%s, %s}, %s", lo.c_str(), hi.c_str(), v.c_str()));
        I(fmt("shfl.sync.bfly.b32 %s, %s, %d, 31, -1", lo2.c_str(), lo.c_str(), lanemask));
        I(fmt("shfl.sync.bfly.b32 %s, %s, %d, 31, -1", hi2.c_str(), hi.c_str(), lanemask));
        I(fmt("mov.b64 %s, {%s, %s}", d.c_str(), lo2.c_str(), hi2.c_str()));
        return d;
    }
    std::string pcoef(uint32_t off) {
        const std::string c = coefs(off, 1)[0];
        return ds_ ? ds_to(c) : c;
    }

    void flush_probes() {
        const int n = static_cast<int>(pending_.size());
        if (n == 0) return;
        int k = 0;
        while ((1 << k) < n) ++k;
        std::vector<std::string> vals;
        for (const auto& q : pending_) vals.push_back(q.v);
        while (static_cast<int>(vals.size()) < (1 << k)) vals.push_back(pzero());
        for (int st = 0; st < k; ++st) {
            const int m = 16 >> st;
            std::string t = R32(), b = P();
            I(fmt("and.b32 %s, %s, %d", t.c_str(), lane_.c_str(), m));
            I(fmt("setp.ne.u32 %s, %s, 0", b.c_str(), t.c_str()));
            const size_t half = vals.size() / 2;
            std::vector<std::string> nv;
            for (size_t i = 0; i < half; ++i) {
                const std::string keep = psel(vals[half + i], vals[i], b);
                const std::string send = psel(vals[i], vals[half + i], b);
                nv.push_back(padd(keep, pshfl(send, m)));
            }
            vals.swap(nv);
        }
        std::string v = vals[0];
        for (int st = k; st < 5; ++st) v = padd(v, pshfl(v, 16 >> st));
        // writer lanes and their probe
        const int lowbits = 5 - k;
        std::string pl = R32(), lo = R32(), w = P(), pin = P();
        I(fmt("shr.u32 %s, %s, %d", pl.c_str(), lane_.c_str(), lowbits));
        I(fmt("and.b32 %s, %s, %d", lo.c_str(), lane_.c_str(), (1 << lowbits) - 1));
        I(fmt("setp.eq.u32 %s, %s, 0", w.c_str(), lo.c_str()));
        I(fmt("setp.lt.and.u32 %s, %s, %d, %s", pin.c_str(), pl.c_str(), n, w.c_str()));
        std::string c = pcoef(pending_[0].coef);
        std::string off = R32();
        I(fmt("mov.u32 %s, %d", off.c_str(), pending_[0].slot * 8));
        for (int i = 1; i < n; ++i) {
            std::string pi = P(), no = R32();
            I(fmt("setp.eq.u32 %s, %s, %d", pi.c_str(), pl.c_str(), i));
            c = psel(pcoef(pending_[i].coef), c, pi);
            I(fmt("selp.b32 %s, %d, %s, %s", no.c_str(), pending_[i].slot * 8, off.c_str(), pi.c_str()));
            off = no;
        }
        std::string ad = R32(), cur = D(), nxt = D();
        I(fmt("add.u32 %s, %s, %s", ad.c_str(), paccW_.c_str(), off.c_str()));
        if (f64_ || ds_) {
            I(fmt("@%s ld.shared.f64 %s, [%s]", pin.c_str(), cur.c_str(), ad.c_str()));
            I(fmt("@%s fma.rn.f64 %s, %s, %s, %s", pin.c_str(), nxt.c_str(), v.c_str(), c.c_str(), cur.c_str()));
        } else {
            std::string vf = mul(v, c), dv = D();
            I(fmt("cvt.f64.f32 %s, %s", dv.c_str(), vf.c_str()));
            I(fmt("@%s ld.shared.f64 %s, [%s]", pin.c_str(), cur.c_str(), ad.c_str()));
            I(fmt("@%s add.rn.f64 %s, %s, %s", pin.c_str(), nxt.c_str(), cur.c_str(), dv.c_str()));
        }
        I(fmt("@%s st.shared.f64 [%s], %s", pin.c_str(), ad.c_str(), nxt.c_str()));
        pending_.clear();
    }
    std::string shfl(const std::string& v, int lanemask) {
        std::string d = A();
        if (f64_) {
            std::string lo = R32(), hi = R32(), lo2 = R32(), hi2 = R32();
            I(fmt("mov.b64 {%s, %s}, %s", lo.c_str(), hi.c_str(), v.c_str()));
            I(fmt("shfl.sync.bfly.b32 %s, %s, %d, 31, -1", lo2.c_str(), lo.c_str(), lanemask));
            I(fmt("shfl.sync.bfly.b32 %s, %s, %d, 31, -1", hi2.c_str(), hi.c_str(), lanemask));
            I(fmt("mov.b64 %s, {%s, %s}", d.c_str(), lo2.c_str(), hi2.c_str()));
        } else {
            std::string r = R32(), r2 = R32();
            I(fmt("mov.b32 %s, %s", r.c_str(), v.c_str()));
            I(fmt("shfl.sync.bfly.b32 %s, %s, %d, 31, -1", r2.c_str(), r.c_str(), lanemask));
            I(fmt("mov.b32 %s, %s", d.c_str(), r2.c_str()));
        }
        return d;
    }

    // Two-target dense gate over the whole tile in shared memory
    // (tile_smem_op / small_apply of device.cuh): quads of amplitudes that
    // differ in tile positions t0 and t1, register controls as a store
    // predicate, controls outside the tile as a uniform skip.
    void smem_step(const StepDesc& sd, const std::string& base, const std::string& sbase) {
        for (int oi = 0; oi < sd.op_count; ++oi) {
            const KOp& o = hp_.ops[sd.op_begin + oi];
            note("shared-memory step: two-target dense gate");
            const std::string lskip = L();
            if (o.cthr) {
                std::string t = R64(), p = P();
                I(fmt("and.b64 %s, %s, %llu", t.c_str(), base.c_str(), static_cast<unsigned long long>(o.cthr)));
                I(fmt("setp.ne.u64 %s, %s, %llu", p.c_str(), t.c_str(), static_cast<unsigned long long>(o.cthr)));
                I(fmt("@%s bra %s", p.c_str(), lskip.c_str()));
            }
            const std::vector<std::string> m = coefs(o.coef, 32);
            std::vector<std::string> nm(16);
            for (int e = 0; e < 16; ++e) nm[e] = neg(m[2 * e + 1]);
            const int lo = o.t0 < o.t1 ? o.t0 : o.t1, hi = o.t0 < o.t1 ? o.t1 : o.t0;
            const uint32_t d0 = tile_weight(o.t0, padu_) * es_, d1 = tile_weight(o.t1, padu_) * es_;
            const int iters = (1 << (T_ - 2)) / NT_;
            for (int k = 0; k < iters; ++k) {
                // i = the quad's index with zeros at lo and hi
                std::string qd = R32();
                I(fmt("add.u32 %s, %s, %d", qd.c_str(), tid_.c_str(), k * NT_));
                std::string i = qd;
                for (int pos : {lo, hi}) {
                    std::string h = R32(), h2 = R32(), l = R32(), n = R32();
                    I(fmt("shr.b32 %s, %s, %d", h.c_str(), i.c_str(), pos));
                    I(fmt("shl.b32 %s, %s, %d", h2.c_str(), h.c_str(), pos + 1));
                    I(fmt("and.b32 %s, %s, %u", l.c_str(), i.c_str(), (1u << pos) - 1));
                    I(fmt("or.b32 %s, %s, %s", n.c_str(), h2.c_str(), l.c_str()));
                    i = n;
                }
                std::string pc;
                if (o.creg) {
                    std::string t = R32();
                    pc = P();
                    I(fmt("and.b32 %s, %s, %u", t.c_str(), i.c_str(), o.creg));
                    I(fmt("setp.eq.u32 %s, %s, %u", pc.c_str(), t.c_str(), o.creg));
                }
                // tile-layout byte address of i; i has zeros at t0 and t1, so
                // the quad's other members add the constants d0, d1, d0 + d1
                std::string t5 = R32(), t8 = R32(), t11 = R32(), sm = R32(), sm2 = R32(), off = R32(), ad = R32();
                I(fmt("shr.b32 %s, %s, 5", t5.c_str(), i.c_str()));
                I(fmt("shr.b32 %s, %s, 8", t8.c_str(), i.c_str()));
                I(fmt("shr.b32 %s, %s, 11", t11.c_str(), i.c_str()));
                I(fmt("add.u32 %s, %s, %s", sm.c_str(), t5.c_str(), t8.c_str()));
                I(fmt("add.u32 %s, %s, %s", sm2.c_str(), sm.c_str(), t11.c_str()));
                I(fmt("mad.lo.u32 %s, %s, %u, %s", off.c_str(), sm2.c_str(), padu_, i.c_str()));
                I(fmt("mad.lo.u32 %s, %s, %d, %s", ad.c_str(), off.c_str(), es_, sbase.c_str()));
                const uint32_t dx[4] = {0u, d0, d1, d0 + d1};
                for (int st = 0; st < NS_; ++st) {
                    Cx in[4];
                    for (int v = 0; v < 4; ++v) in[v] = load_amp(ad, st * tileB_ + dx[v]);
                    Cx out[4];
                    for (int r = 0; r < 4; ++r) {  // quad_dense of policy.cuh
                        const int b0 = 8 * r;
                        std::vector<std::pair<std::string, std::string>> tr, ti;
                        for (int c = 0; c < 4; ++c) {
                            const std::string& mr = m[b0 + 2 * c];
                            const std::string& mi = m[b0 + 2 * c + 1];
                            tr.push_back({mr, in[c].x});
                            tr.push_back({nm[4 * r + c], in[c].y});
                            ti.push_back({mr, in[c].y});
                            ti.push_back({mi, in[c].x});
                        }
                        out[r] = {dot(tr), dot(ti)};
                    }
                    for (int v = 0; v < 4; ++v) store_amp(ad, st * tileB_ + dx[v], out[v], pc);
                }
            }
            lab(lskip);
            I("bar.sync 0");
        }
    }

    void round(const StepDesc& sd, const std::string& base, const std::string& sbase) {
        bool need_g = false;
        for (int oi = 0; oi < sd.op_count; ++oi)
            if (hp_.ops[sd.op_begin + oi].flags & (F_TCTRL | F_TPAR)) need_g = true;
        // the thread's tile-layout byte address in this slot; register j adds offb(j)
        std::vector<uint32_t> tsw(T_ - R_);
        for (int k = 0; k < T_ - R_; ++k) tsw[k] = static_cast<uint32_t>(sd.tsw[k]) * es_;
        std::string psb = R32();
        I(fmt("add.u32 %s, %s, %s", psb.c_str(), sum32(tid_, T_ - R_, tsw).c_str(), sbase.c_str()));
        // 8-byte elements with tile position 0 in register bit r0: registers j
        // and j | 1 << r0 are adjacent, accessed 16 bytes at a time
        int r0 = -1;
        if (es_ == 8)
            for (int k = 0; k < R_; ++k)
                if (sd.rpos[k] == 0) r0 = k;
        std::string gthr;
        if (need_g) {
            std::vector<uint64_t> tg(T_ - R_);
            for (int k = 0; k < T_ - R_; ++k) tg[k] = 1ULL << sd.tglob[k];
            std::string td = deposit64(tid_, T_ - R_, tg);
            gthr = R64();
            I(fmt("or.b64 %s, %s, %s", gthr.c_str(), base.c_str(), td.c_str()));
        }
        auto offb = [&](int j) {
            uint32_t o = 0;
            for (int k = 0; k < R_; ++k)
                if ((j >> k) & 1) o += static_cast<uint32_t>(sd.rsw[k]) * es_;
            return o;
        };
        note("round: loads");
        A_.assign(NS_, std::vector<Cx>(NA_));
        for (int j = 0; j < NA_; ++j) {
            if (r0 >= 0) {
                if ((j >> r0) & 1) continue;
                const int j1 = j | (1 << r0);
                for (int s = 0; s < NS_; ++s) {
                    Cx a{A(), A()}, b{A(), A()};
                    I(fmt("ld.shared.v4.f32 {%s, %s, %s, %s}, [%s+%u]", a.x.c_str(), a.y.c_str(), b.x.c_str(),
                          b.y.c_str(), psb.c_str(), s * tileB_ + offb(j)));
                    A_[s][j] = a;
                    A_[s][j1] = b;
                }
                continue;
            }
            for (int s = 0; s < NS_; ++s) A_[s][j] = load_amp(psb, s * tileB_ + offb(j));
        }
        ph_on_ = false;
        q_.clear();
        flip_.assign(R_, std::string());
        for (int oi = 0; oi < sd.op_count; ++oi) {
            const KOp& o = hp_.ops[sd.op_begin + oi];
            const std::string ctl = (o.flags & F_TCTRL) ? ctl_pred(o, gthr) : "";
            if (o.kind == K_X && !ctl.empty() && o.creg == 0) {
                add_flip(o.t0, ctl);  // thread-controlled X: a pending flip of the thread's bit t0
                continue;
            }
            // register controls, parities and targets whose meaning a flip changes
            uint32_t need = o.creg;
            if (o.kind == K_DIAG) need |= o.preg | ((o.flags & F_ONEBIT) ? (1u << o.t0) : 0u);
            if (o.kind == K_Y || o.kind == K_HAD) need |= 1u << o.t0;
            if (o.kind == K_SWAP && o.creg) need |= (1u << o.t0) | (1u << o.t1);
            if (o.kind == K_PROBE) need |= o.xreg | o.preg;
            if (o.kind == K_DIAGR) need |= (1u << R_) - 1;  // its entries are per register index
            for (int t = 0; t < R_; ++t)
                if ((need >> t) & 1) {
                    if (!flip_[t].empty()) note(fmt("materialize flip %d for kind %d", t, o.kind));
                    materialize(t);
                }
            note(fmt("op kind %d t0 %d%s", o.kind, o.t0, ctl.empty() ? "" : " thread-controlled"));
            if (o.kind == K_PROBE) op_probe(o, gthr, ctl);
            else if (o.kind == K_DIAG) op_diag(o, gthr, ctl);
            else if (o.kind == K_DIAGR) op_diagr(o);
            else op_gate(o, ctl);
        }
        flush_probes();
        note("round end: uniform phase, stores");
        // the round's uniform phase (reg_finish_phase)
        if (!q_.empty()) {
            std::string q1 = R32(), q2 = R32(), s1 = P(), s2 = P();
            I(fmt("and.b32 %s, %s, 1", q1.c_str(), q_.c_str()));
            I(fmt("and.b32 %s, %s, 2", q2.c_str(), q_.c_str()));
            I(fmt("setp.ne.u32 %s, %s, 0", s1.c_str(), q1.c_str()));
            I(fmt("setp.ne.u32 %s, %s, 0", s2.c_str(), q2.c_str()));
            if (ph_on_) {
                ph_ = rot_q(ph_, s1, s2);
            } else {
                for (int s = 0; s < NS_; ++s)
                    for (int j = 0; j < NA_; ++j) A_[s][j] = rot_q(A_[s][j], s1, s2);
            }
        }
        if (ph_on_) {
            const std::string nfi = neg(ph_.y);
            for (int s = 0; s < NS_; ++s)
                for (int j = 0; j < NA_; ++j) A_[s][j] = phase(A_[s][j], ph_.x, ph_.y, nfi);
        }
        // a pending flip of bit t: register j holds logical j ^ (1 << t), whose
        // address is j's plus rsw[t] (bit t of j clear) or minus it (set)
        if (r0 >= 0) materialize(r0);  // pairs are stored as they are
        std::vector<int> fl;
        std::vector<std::string> fpos, fneg;
        for (int t = 0; t < R_; ++t) {
            if (flip_[t].empty()) continue;
            const uint32_t w = static_cast<uint32_t>(sd.rsw[t]) * es_;
            std::string vp = R32(), vn = R32();
            I(fmt("selp.b32 %s, %u, 0, %s", vp.c_str(), w, flip_[t].c_str()));
            I(fmt("selp.b32 %s, %u, 0, %s", vn.c_str(), 0u - w, flip_[t].c_str()));
            fl.push_back(t);
            fpos.push_back(vp);
            fneg.push_back(vn);
        }
        std::map<int, std::string> fbase;  // flip-bit pattern of j -> store base
        auto store_base = [&](int j) {
            int pat = 0;
            for (size_t x = 0; x < fl.size(); ++x) pat |= ((j >> fl[x]) & 1) << x;
            auto it = fbase.find(pat);
            if (it != fbase.end()) return it->second;
            std::string acc = psb;
            for (size_t x = 0; x < fl.size(); ++x) {
                std::string n = R32();
                I(fmt("add.u32 %s, %s, %s", n.c_str(), acc.c_str(), ((pat >> x) & 1) ? fneg[x].c_str() : fpos[x].c_str()));
                acc = n;
            }
            fbase[pat] = acc;
            return acc;
        };
        for (int j = 0; j < NA_; ++j) {
            if (r0 >= 0) {
                if ((j >> r0) & 1) continue;
                const int j1 = j | (1 << r0);
                const std::string ad = store_base(j);
                for (int s = 0; s < NS_; ++s)
                    I(fmt("st.shared.v4.f32 [%s+%u], {%s, %s, %s, %s}", ad.c_str(), s * tileB_ + offb(j),
                          A_[s][j].x.c_str(), A_[s][j].y.c_str(), A_[s][j1].x.c_str(), A_[s][j1].y.c_str()));
                continue;
            }
            const std::string ad = store_base(j);
            for (int s = 0; s < NS_; ++s) store_amp(ad, s * tileB_ + offb(j), A_[s][j]);
        }
        I("bar.sync 0");
    }

    // pending per-thread flips of register bits (thread-controlled X)
    void add_flip(int t, const std::string& p) {
        if (flip_[t].empty()) {
            flip_[t] = p;
            return;
        }
        std::string q = P();
        I(fmt("xor.pred %s, %s, %s", q.c_str(), flip_[t].c_str(), p.c_str()));
        flip_[t] = q;
    }
    void materialize(int t) {
        if (flip_[t].empty()) return;
        const std::string p = flip_[t];
        flip_[t].clear();
        for (int j : pairs(t, 0))
            for (int s = 0; s < NS_; ++s) {
                const Cx a = A_[s][j], b = A_[s][j | (1 << t)];
                A_[s][j] = {sel(b.x, a.x, p), sel(b.y, a.y, p)};
                A_[s][j | (1 << t)] = {sel(a.x, b.x, p), sel(a.y, b.y, p)};
            }
    }

    // ---------------------------------------------------------------- state
    const HostPlan& hp_;
    const PassDesc& pd_;
    JitShape sh_;
    bool f64_, ds_;
    const char* ft_;
    int es_, cb_, T_, R_, NT_, NA_, NW_, PER_, NS_, np_, H_, RUNS_;
    uint32_t padu_, runB_, tileB_, slotB_;
    bool bc_ = false;  // bounds-checked accesses
    bool in_pair_ = false, out_pair_ = false;  // float pairs in global memory before / after the pass
    bool bulk_out_ = true;                     // write-back by bulk stores of the slot
    std::string smend_, gend_[2];
    bool pc_ = false;  // coefficients from the parameter block p_cblob
    uint32_t cmin_ = 0, cmax_ = 0;
    static constexpr uint32_t kMaxBlob = 16384;  // bytes of coefficients in the kernel parameters
    std::string body_;
    int nr_ = 0, nrd_ = 0, nh_ = 0, np_reg_ = 0, na_ = 0, nd_ = 0, nl_ = 0;
    std::map<double, std::string> consts_;
    std::string tid_, bid64_, nbid64_, stg_[2], ntiles_, coef0_, cstrideB_, ishift_, active_, hasact_, smb_;
    std::string gtidB_, stidB_, lane_, paccB_, paccW_, perTile_, partial_, coefp_;
    std::string status_, waitns_, extra_, iss_, t0_, runG_, runS_, runb_, txb_, mbarB_;
    struct Pending {
        std::string v;
        int slot;
        uint32_t coef;
    };
    std::vector<Pending> pending_;
    std::vector<std::vector<Cx>> A_;
    std::vector<std::string> flip_;
    bool ph_on_ = false;
    Cx ph_;
    std::string q_;
};

}  // namespace

namespace {
template <class T>
void put(std::string* k, const T& v) {
    k->append(reinterpret_cast<const char*>(&v), sizeof(T));
}
}  // namespace

bool jit_pass_key(const HostPlan& hp, int pi, const JitShape& sh, std::string* key, std::string* why) {
    if (pi < 0 || pi >= static_cast<int>(hp.passes.size())) {
        if (why) *why = "pass index out of range";
        return false;
    }
    Gen g(hp, pi, sh);
    if (!g.supported(why)) return false;
    // every field the generator reads, explicitly (no struct padding)
    const PassDesc& pd = hp.passes[pi];
    std::string& k = *key;
    k.clear();
    put(&k, hp.arith);
    put(&k, hp.T);
    put(&k, hp.R);
    put(&k, sh.nstates);
    put(&k, sh.nb);
    put(&k, sh.minb);
    put(&k, static_cast<int>(g.param_coefs()));
    put(&k, sh.bounds);
    put(&k, static_cast<int>(g.in_pairs()));
    put(&k, static_cast<int>(g.out_pairs()));
    put(&k, pd.L);
    put(&k, pd.H);
    put(&k, pd.step_count);
    put(&k, sh.nstates == 2 ? pd.nprobe : 0);
    k.append(reinterpret_cast<const char*>(pd.tq), sizeof pd.tq);
    for (int si = 0; si < pd.step_count; ++si) {
        const StepDesc& sd = hp.steps[pd.step_begin + si];
        put(&k, sd.type);
        put(&k, sd.op_count);
        k.append(reinterpret_cast<const char*>(sd.tglob), sizeof sd.tglob);
        k.append(reinterpret_cast<const char*>(sd.rsw), sizeof sd.rsw);
        k.append(reinterpret_cast<const char*>(sd.tsw), sizeof sd.tsw);
        for (int oi = 0; oi < sd.op_count; ++oi) {
            const KOp& o = hp.ops[sd.op_begin + oi];
            put(&k, o.kind);
            put(&k, o.flags);
            put(&k, o.special);
            put(&k, o.t0);
            put(&k, o.t1);
            put(&k, o.probe);
            put(&k, o.creg);
            put(&k, o.preg);
            put(&k, o.cthr);
            put(&k, o.pthr);
            put(&k, o.coef);
            put(&k, o.xreg);
            put(&k, o.k);
            k.append(reinterpret_cast<const char*>(o.tk), sizeof o.tk);
        }
    }
    return true;
}

bool jit_pass_coef_block(const HostPlan& hp, int pi, const JitShape& sh, uint32_t* cmin, uint32_t* cmax) {
    if (pi < 0 || pi >= static_cast<int>(hp.passes.size())) return false;
    Gen g(hp, pi, sh);
    if (!g.param_coefs()) return false;
    *cmin = g.cmin();
    *cmax = g.cmax();
    return true;
}

size_t jit_smem_bytes(const HostPlan& hp, const JitShape& sh, int nprobe) {
    const int es = hp.arith == QFVM_C64 ? 8 : 16;
    const size_t tileB = static_cast<size_t>(tile_elems(hp.T, es)) * es;
    const size_t nw = static_cast<size_t>(1 << (hp.T - hp.R)) / 32;
    const size_t np = sh.nstates == 2 ? static_cast<size_t>(nprobe) : 0;
    return static_cast<size_t>(sh.nb) * sh.nstates * tileB + nw * np * 8 + 8 * static_cast<size_t>(sh.nb);
}

bool jit_pass_ptx(const HostPlan& hp, int pi, const JitShape& sh, const std::string& entry, std::string* ptx,
                  std::string* why) {
    if (pi < 0 || pi >= static_cast<int>(hp.passes.size())) {
        if (why) *why = "pass index out of range";
        return false;
    }
    Gen g(hp, pi, sh);
    if (!g.supported(why)) return false;
    *ptx = g.emit(entry);
    return true;
}

}  // namespace qsv
