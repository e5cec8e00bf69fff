"""Reader of CONTACT's stand-alone input files for module 3 (the ".inp" format).

Turns the cases of a module-3 input file into case dicts for
contact_gb300.setup_case (and the oracle), so that the reference's own example and
performance inputs replay through this library.  It follows the reading order of the
stand-alone program's input routine (src/m_sinput.f90:34-317: control digits, solver,
kinematics, friction, rolling step, material, potential contact, geometry) and its line
conventions (src/m_readline.f90:36-288): '%' starts a comment, a data line ends at its first
non-numeric word, required values may continue on the next lines, Fortran number forms
('.1-07', '1d0'), angles with a 'd' (degrees) or 'r' suffix.

Values that a case does not repeat keep their previous value, as in the program: a case
with G=1 keeps the solver settings, D=0 the potential contact, Z<2 the geometry.

Supported: control digits of module 3, creepages or total forces prescribed (F=0, 1, 2),
with Coulomb or falling friction (L=0, 2, 3, 4; V=0), elastic materials (two different bodies: keys poiss2, gg2)
(M=0) or elastic bodies with an elastic interfacial layer (M=4 with TAU_C0 = 0: keys mater, gg3,
laythk, tau_c0, k_tau), no thin-sheet, heat or extra-rigid-slip inputs; potential contact
IPOTCN -3..-1 and 1..4; geometry IBASE 1 (quadratic), 2 (circular in x, tabulated in y),
3 (sines in x) and 9 (element-wise), planform IPLAN 1; subsurface points (S digit, key
'subs'), previous time instances (P digit, key 'pvtime').  IBASE 2 and 3 are evaluated here
(set_norm_rhs, src/m_sdis.f90:321-494) and handed on element-wise.  A case that uses
anything else is returned with an 'unsupported' entry and ends the reading.
"""
import math
import re

import numpy as np

__all__ = ["read_inp", "materialize", "parse_number"]

_FORTRAN_EXP = re.compile(r"^([+-]?(?:\d+\.?\d*|\.\d+))([+-]\d+)$")


def parse_number(word, angle=False):
    """A Fortran-style real: 1.5, .1-07 (= 0.1e-7), 2.5d0, 1e-5; with angle, a trailing 'd'
    means degrees and 'r' radians."""
    w = word.strip().lower()
    deg = False
    if angle and w and w[-1] in "dr":
        deg = w[-1] == "d"
        w = w[:-1]
    w = w.replace("d", "e")
    m = _FORTRAN_EXP.match(w)
    if m:
        w = m.group(1) + "e" + m.group(2)
    v = float(w)
    return v * math.pi / 180.0 if deg else v


class _Lines:
    """Data lines of an input file: comments removed, blank lines skipped."""

    def __init__(self, text):
        self.lines = []
        for ln in text.splitlines():
            body = ln.split("%", 1)[0].replace(",", " ").strip()
            if body:
                self.lines.append(body.split())
        self.pos = 0

    def eof(self):
        return self.pos >= len(self.lines)

    def read(self, types):
        """Read values of the given types ('i' int, 'd' real, 'a' angle; upper case optional)
        like the program's readline: words of a line until the first non-number, more lines
        while the required values are not complete."""
        nreq = sum(1 for t in types if t.islower())
        vals = []
        while len(vals) < nreq:
            if self.eof():
                raise ValueError("input ends while reading %r" % types)
            words = self.lines[self.pos]
            self.pos += 1
            for w in words:
                if len(vals) >= len(types):
                    break
                t = types[len(vals)].lower()
                try:
                    v = int(w) if t == "i" else parse_number(w, angle=(t == "a"))
                except ValueError:
                    break
                vals.append(v)
        return vals

    def read_array(self, n, kind="d"):
        """n values over as many lines as needed (read1darr, src/m_readline.f90:292-446)."""
        vals = []
        while len(vals) < n:
            if self.eof():
                raise ValueError("input ends while reading %d values" % n)
            words = self.lines[self.pos]
            self.pos += 1
            for w in words:
                if len(vals) >= n:
                    break
                try:
                    vals.append(int(w) if kind == "i" else parse_number(w))
                except ValueError:
                    break
        return vals


def _digits(value, names):
    """Unpack control digits from the right (ic_unpack, src/m_hierarch_data.f90:1128-1216)."""
    out = {}
    v = int(value)
    for name in reversed(names):
        out[name] = v % 10
        v //= 10
    return out


def _ibase2_h(prm, nn, x, y):
    """IBASE 2: a table in y (linear between the nn points y1 + k dy1), plus the circle
    (x - xm)^2 / (2 rm) in x (set_norm_rhs, src/m_sdis.f90:358-381)."""
    xm, rm, y1, dy1 = prm[0], prm[1], prm[2], prm[3]
    tab = prm[4:]
    yn = y1 + (nn - 1) * dy1
    h = np.empty_like(x)
    for i in range(x.size):
        if y[i] < y1:
            yleft, mleft = y1, 1
        elif y[i] >= yn:
            yleft, mleft = yn - dy1, nn - 1
        else:
            mleft = int((y[i] - y1) / dy1) + 1
            yleft = y1 + (mleft - 1) * dy1
        rc = (tab[mleft] - tab[mleft - 1]) / dy1
        h[i] = tab[mleft - 1] + rc * (y[i] - yleft) + (x[i] - xm) ** 2 / (2.0 * rm)
    return h


def _ibase3_h(p, x, y):
    """IBASE 3: two sines in x and a quadratic (set_norm_rhs, src/m_sdis.f90:382-389)."""
    return (p[0] * np.sin(p[1] * (x - p[2])) - p[3] * np.sin(p[4] * (x - p[5])) + x ** 2 / p[6] + y ** 2 / p[7])


def _grid_centres(pot):
    """Element centres of a non-Hertzian potential contact (potcon_fill,
    src/m_hierarch_data.f90:1801-1861), element index ii = ix + (iy-1) mx."""
    ip, mx, my = pot["ipotcn"], pot["mx"], pot["my"]
    a, b, c, d = pot["prm"]
    if ip == 1:
        xl, yl, dx, dy = a, b, c, d
        xc1, yc1 = xl + 0.5 * dx, yl + 0.5 * dy
    elif ip == 2:
        xl, yl, xh, yh = a, b, c, d
        dx, dy = (xh - xl) / mx, (yh - yl) / my
        xc1, yc1 = xl + 0.5 * dx, yl + 0.5 * dy
    elif ip == 3:
        xc1, yc1, dx, dy = a, b, c, d
    else:
        xc1, yc1, xcm, ycm = a, b, c, d
        dx = (xcm - xc1) / max(1, mx - 1)
        dy = (ycm - yc1) / max(1, my - 1)
    x = xc1 + dx * np.arange(mx)
    y = yc1 + dy * np.arange(my)
    X, Y = np.meshgrid(x, y)
    return X.ravel(), Y.ravel()


def read_inp(text):
    """Module-3 cases of an input file (its text) as a list of case dicts."""
    L = _Lines(text)
    st = dict(maxgs=999, maxin=100, maxnr=30, maxout=1, eps=1e-6, gd=None, veloc=1.0, chi=0.0, dq=1.0,
              fstat=0.3, poiss=(0.28, 0.28), gg=(82000.0, 82000.0), pot=None, geom=None)
    cases = []
    while not L.eof():
        module = L.read("i")[0]
        if module == 0:
            break
        if module != 3:
            cases.append({"unsupported": "module %d" % module})
            break
        c = {}
        pb = _digits(L.read("i")[0], "CPBTNFS")
        vl = L.read("iI")
        vd = _digits(vl[0], "VLDCMZE")
        xh = _digits(L.read("i")[0], "XHGIAOWR")
        if xh["X"] >= 1:
            L.read("iI")
        bad = []
        if vd["V"] != 0 or vd["L"] not in (0, 1, 2, 3, 4):
            bad.append("friction law V=%d L=%d" % (vd["V"], vd["L"]))
        if vd["M"] not in (0, 4) or pb["B"] == 1:
            bad.append("material M=%d B=%d" % (vd["M"], pb["B"]))
        if xh["H"] != 0 or vd["E"] != 0:
            bad.append("heat or extra rigid slip inputs")
        if len(vl) >= 2 and vl[1] % 10 >= 2:
            bad.append("damping inputs")
        if pb["P"] == 3:
            bad.append("previous time instance kept as is (P=3)")
        if bad:
            cases.append({"unsupported": "; ".join(bad)})
            break
        g = xh["G"]
        if g != 1:
            v = L.read("iiiidI")
            st.update(maxgs=v[0], maxin=v[1], maxnr=v[2], maxout=v[3], eps=v[4], gausei=g)
            if g in (2, 3):
                v = L.read("ddid")
                st.update(relax=dict(omegah=v[0], omegas=v[1], inislp=v[2], omgslp=v[3]))
            if g == 4:
                v = L.read("id")
                st.update(relax=dict(st.get("relax") or {}, inislp=v[0], omgslp=v[1]))
            if g == 5:
                v = L.read("ddiddddd")
                st["gd"] = dict(fdecay=v[0], betath=v[1], kdowfb=v[2], d_ifc=v[3], d_lin=v[4], d_cns=v[5],
                                d_slp=v[6], pow_s=v[7])
        kin = L.read("ddddDD")
        if pb["N"] == 0:
            c["pen"] = kin[0]
        else:
            c["fn"] = kin[0]
        # m_sinput.f90:720-733: F=0 creepages, F=1 Fx/(mu Fn) and ceta, F=2 Fx/(mu Fn) and Fy/(mu Fn)
        if pb["F"] == 0:
            c["cksi"], c["ceta"] = kin[1], kin[2]
        elif pb["F"] == 1:
            c["fxrel"], c["ceta"] = kin[1], kin[2]
        else:
            c["fxrel"], c["fyrel"] = kin[1], kin[2]
        c["cphi"] = kin[3]
        if pb["F"] != 0:
            c["force3"] = pb["F"]
        if vd["L"] == 0:
            st["fstat"] = L.read("dd")[0]
            st["flaw"] = None
        elif vd["L"] in (2, 3, 4):
            # falling friction (fric_input, src/m_friclaw.f90:622-868): fkin, f1, sabsh1, f2,
            # sabsh2, then the friction memory memdst, mem_s0
            st["flaw"] = dict(frclaw=vd["L"], flaw=L.read("ddddd"), mem=L.read("dd"))
        if vd["C"] in (2, 3, 4, 9):
            if pb["T"] in (2, 3):
                v = L.read("addD")
                st.update(chi=v[0], dq=v[1], veloc=v[2])
            if vd["C"] != 2:
                cases.append({"unsupported": "influence coefficients C=%d (only piecewise constant, C=2)" % vd["C"]})
                break
            v = L.read("dddd")
            st.update(poiss=(v[0], v[1]), gg=(v[2], v[3]))
            if vd["M"] == 4:
                # the interfacial layer (m_sinput.f90:942-955): GG3, LAYTHK, TAU_C0, K_TAU;
                # TAU_C0 >= 1e10 means no yield limit
                v = L.read("dddd")
                st["layer"] = dict(gg3=v[0], laythk=v[1], tau_c0=0.0 if v[2] >= 1e10 else v[2], k_tau=v[3])
        if vd["M"] == 4 and (st.get("layer") is None or st["layer"]["tau_c0"] > 1e-10):
            cases.append({"unsupported": "plastic interfacial layer (M=4, TAU_C0 > 0)"})
            break
        if vd["D"] == 2:
            ip = L.read("i")[0]
            if -3 <= ip <= -1:
                v = L.read("iiddd")
                st["pot"] = dict(ipotcn=ip, mx=v[0], my=v[1], prm=v[2:5])
            elif 1 <= ip <= 4:
                v = L.read("iidddd")
                st["pot"] = dict(ipotcn=ip, mx=v[0], my=v[1], prm=v[2:6])
            else:
                cases.append({"unsupported": "potential contact IPOTCN=%d" % ip})
                break
        pot = st["pot"]
        if vd["Z"] >= 2:
            if pot["ipotcn"] < 0:
                st["geom"] = None
            else:
                ib, ipl = L.read("ii")
                if ipl != 1:
                    cases.append({"unsupported": "planform IPLAN=%d" % ipl})
                    break
                if ib == 1:
                    st["geom"] = ("prmudf", L.read_array(6))
                elif ib == 2:
                    v = L.read("idddd")
                    st["geom"] = ("ibase2", [float(v[0])] + list(v[1:5]) + L.read_array(v[0]))
                elif ib == 3:
                    st["geom"] = ("ibase3", L.read_array(8))
                elif ib == 9:
                    st["geom"] = ("h", np.asarray(L.read_array(pot["mx"] * pot["my"])))
                else:
                    cases.append({"unsupported": "geometry IBASE=%d" % ib})
                    break
        c.update(tang=pb["T"], norm=pb["N"], bound=pb["B"], pvtime=pb["P"], iestim=xh["I"],
                 gausei=st.get("gausei", 0), maxgs=st["maxgs"], maxin=st["maxin"], maxnr=st["maxnr"],
                 maxout=st["maxout"], eps=st["eps"], poiss=st["poiss"][0], gg=st["gg"][0], fstat=st["fstat"],
                 standalone=True,
                 veloc=st["veloc"], ipotcn=pot["ipotcn"], potprm=[pot["mx"], pot["my"]] + list(pot["prm"]))
        if pb["S"] >= 2:
            st["subs"] = _read_subsurface(L, pb["S"], st.get("subs"))
        if pb["S"] >= 1 and st.get("subs"):
            c["subs"] = st["subs"]
        if st["poiss"][0] != st["poiss"][1] or st["gg"][0] != st["gg"][1]:
            c["poiss2"], c["gg2"] = st["poiss"][1], st["gg"][1]
        if vd["M"] == 4:
            c.update(mater=4, **st["layer"])
        if st["gd"] is not None:
            c["gd"] = dict(st["gd"])
        if st.get("relax") is not None and c["gausei"] in (2, 3, 4):
            c.update(st["relax"])
        if st.get("flaw"):
            f = st["flaw"]
            c.update(frclaw=f["frclaw"], flaw=list(f["flaw"]), memdst=f["mem"][0], mem_s0=f["mem"][1])
            c["fstat"] = f["flaw"][0] + f["flaw"][1] + f["flaw"][3]
        if pb["T"] in (2, 3):
            c["dq"] = st["dq"]
            if abs(st["chi"]) > 1e-12:
                c["chi"] = st["chi"]
        if pot["ipotcn"] >= 1 and st["geom"] is not None:
            key, val = st["geom"]
            c[key] = np.asarray(val, dtype=np.float64) if key == "h" else list(val)
        cases.append(materialize(c))
    return cases


def _read_subsurface(L, sdigit, prev):
    """Subsurface points of a case (subsurf_input, src/m_subsurf.f90:65-298): the A, O digits
    for the results and, for S=3, blocks until ISUBS = 0.  Each block a dict: isubs and
    either the element selection ('ix', 'iy': 1-based column and row numbers, isubs 1-3 and
    5-7; None for all) with depths 'z', or coordinate lists 'x', 'y', 'z' (isubs 9).  S=2 keeps
    the previous blocks."""
    L.read("ii")
    if sdigit < 3:
        return prev
    blocks = []
    isubs = L.read("i")[0]
    while isubs >= 1:
        b = {"isubs": isubs}
        if isubs in (1, 5):
            b["ix"] = b["iy"] = None
        elif isubs in (2, 6):
            xl, xinc, xh = L.read("iii")
            yl, yinc, yh = L.read("iii")
            b["ix"] = list(range(xl, xh + 1, max(1, xinc)))
            b["iy"] = list(range(yl, yh + 1, max(1, yinc)))
        elif isubs in (3, 7):
            nx, ny = L.read("ii")
            b["ix"] = sorted(set(int(v) for v in L.read_array(nx)))
            b["iy"] = sorted(set(int(v) for v in L.read_array(ny)))
        if isubs in (1, 2, 3):
            nz, zl, dz = L.read("idd")
            b["z"] = [zl + k * dz for k in range(max(1, nz))]
        elif isubs in (5, 6, 7):
            nz = L.read("i")[0]
            b["z"] = sorted(L.read_array(max(1, nz)))
        elif isubs == 9:
            nx, ny, nz = L.read("iii")
            b["x"] = sorted(L.read_array(max(1, nx)))
            b["y"] = sorted(L.read_array(max(1, ny)))
            b["z"] = sorted(L.read_array(max(1, nz)))
        else:
            raise ValueError("subsurface input option ISUBS=%d" % isubs)
        blocks.append(b)
        isubs = L.read("i")[0]
    return blocks


def materialize(case):
    """Add the element-wise undeformed distance 'h' of a case whose geometry is given as
    IBASE 2 ('ibase2': [nn, xm, rm, y1, dy1, table...]) or IBASE 3 ('ibase3': 8 values)."""
    if "h" in case or not ("ibase2" in case or "ibase3" in case):
        return case
    pr = case["potprm"]
    X, Y = _grid_centres(dict(ipotcn=case["ipotcn"], mx=int(pr[0]), my=int(pr[1]), prm=pr[2:6]))
    if "ibase2" in case:
        g = case["ibase2"]
        h = _ibase2_h(g[1:], int(g[0]), X, Y)
    else:
        h = _ibase3_h(case["ibase3"], X, Y)
    out = dict(case)
    out["h"] = h
    return out
