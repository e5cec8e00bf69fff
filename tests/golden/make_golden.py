"""Extract golden vectors from the reference's own regression outputs.

Reads, as text, output and input files of the CONTACT repository and writes compact JSON
fixtures next to this script:

* testbank/test_table_mx11.ref_fx -> test_table_mx11.json
  output of src/test_table.f90 (3220 Hertzian steady-rolling cases through the
  library API: 11x11 grid, NormCG + SteadyGS, eps 1e-6).  Per case the
  normalised forces Fx/(mu Fn), Fy/(mu Fn), Mz/(mu Fn cp) to 6 decimals and the
  slip percentage.
* examples/tractcurv.ref_out -> tractcurv_series1.json
  first series (cases 1-30) of examples/tractcurv.inp (Hertz a1/aob input, 48x44 grid,
  Coulomb friction, SteadyGS): forces, energy, approach, pmax to 4 digits,
  element counts, iteration counts and the element-division picture.
* examples/cattaneo.ref_out -> cattaneo.json
  examples/cattaneo.inp, 19x19 grid, polyethylene ball on a plane (G 200, nu 0.42, mu 0.4):
  case 1 the Hertzian normal problem (NormCG), case 2 the non-Hertzian quadratic geometry
  with the shift problem (T=1, TangCG) whose tangential forces the reference prescribes
  (F=2) and meets by Newton-Raphson on the shifts; kept: the iterations of that process
  (shifts, relative forces, TangCG iterations), the sensitivities it leaves, forces,
  approach, pmax, element counts and the element-division picture.
* examples/catt_to_cart.inp + catt_to_cart.ref_out -> catt_to_cart_sequence.json
  all 171 cases: three transient sequences (rolling on a fixed grid, shifts on a fixed and
  on a moving grid) continuing from case to case with Fx prescribed: the reader's cases and
  the printed Newton-Raphson rows and counts.
* examples/catt_to_cart.ref_out -> catt_to_cart_case1.json
  case 1 of examples/catt_to_cart.inp, the Cattaneo shift problem on a 34x33 grid with Fx
  prescribed (F=1, TangCG, eps 1e-7): the Newton-Raphson iterations, the sensitivity
  dFx/dcksi, forces, shift, element counts and the element-division picture.

* examples/carter2d.ref_out -> carter2d.json
  examples/carter2d.inp, Carter's two-dimensional steady rolling problem on a 55x1 strip
  (dy 200 mm, SteadyGS, eps 1e-5), printed with its element tables: the approach to 8 digits,
  pn per element after NORM, element codes, px and shift sx after TANG, totals and counts.

* examples/subsurf.ref_subs + subsurf.ref_out -> subsurf.json
  the two solves of examples/subsurf.inp (one 1x1 mm element: the normal problem, then
  steady rolling with Fx prescribed, which the reference solves by ConvexGS and
  Newton-Raphson) with their printed results, and the subsurface elastic field of the second
  one's tractions (pressure 1, traction 0.999):
  displacements, hydrostatic and von Mises stresses and the six stress components at 15
  depths below one point and below a 7x7 subgrid of a 21x21 block, as printed, and the
  printed maxima of both cases (pressure alone and with traction).

* examples/bentall.inp + bentall.ref_out -> bentall.json
  steady rolling of two different materials (coupled normal and tangential problems,
  several outer iterations) on a 216x1 strip at chi = 180 deg with Fx prescribed: the
  reader's six cases, to be replayed in order, and the printed results of cases 2-6.

* examples/spence35.inp + spence35.ref_out -> spence35.json
  Spence's problem in 35 load steps (two materials, coupled problems, each step continuing
  from the previous one, subsurface stresses along one row): the reader's cases, the printed
  outer iterations, totals and counts, and the printed subsurface maxima.

* examples/veldep_fric.inp + veldep_fric.ref_out -> veldep_fric_case1.json
  case 1, steady rolling with an exponential falling friction law (L=4) on a 92x1 strip by
  ConvexGS: the printed iterations on the slip velocity, sweeps, counts and totals.
* examples/tractcurv.inp + tractcurv.ref_out -> tractcurv_series2.json
  the second series (cases 31-60): elastic bodies with an elastic interfacial layer (M=4),
  exponential falling friction with a friction memory, SteadyGS on a 48x44 grid: the reader's
  cases and per case the slip-velocity iterations, counts, iterations, totals and picture.
* testbank/testbank.ref_out -> testbank_case3_subs.json
  case 3: the normal problem of two bodies and the subsurface field at six points in both.
* examples/veldep_fric.inp + veldep_fric.ref_out -> veldep_fric_sequence.json
  all 53 cases (steady rolling, then transient rolling steps continuing from the previous
  time instance): the reader's cases and per case the printed slip-velocity iterations,
  the last solve's sweeps, counts and totals.

* testbank/test_caddon.ref_out -> test_caddon_re1.json
  output of src/test_caddon.f90 for result element 1 (module 3 through the library
  interface in SPCK units: Hertzian 21x33 grid, penetration prescribed, creepage 0.001,
  spin 0.4 rad/m, SteadyGS, eps 1e-4): grid spacing, forces, moment, patch areas, maximum
  pressure and traction, positions and values of the largest tractions.  (Result element 2
  uses a falling friction law and an interfacial layer, outside this library.)

* testbank/contact_nonhz.ref_out -> contact_nonhz_re1.json
  the same call sequence as test_caddon's element 1, printed by the library in CONTACT units
  (mm, N): forces, moment, energy, approach, pmax to 4 digits, element counts, NormCG and
  SteadyGS iterations and the element-division picture.

* testbank/testbank.ref_out -> testbank_cases.json
  cases 1, 7, 10 and 13 of testbank/testbank.inp, the stand-alone program's regression set:
  case 1 the shift problem with prescribed approach (17x17 quadratic geometry, TangCG, eps
  1e-8), case 6 Carter's strip by ConvexGS (G=2) with a rolling step of 5 dx, case 9 steady
  rolling of two different materials (coupled normal and tangential problems), case 7 steady rolling on a 41x41 quadratic geometry (SteadyGS, eps 1e-6), case 10
  the same shift with Fn, Fx and Fy prescribed (F=2, Newton-Raphson on both shifts), case 13
  a shift on a 41x41 Hertzian grid with the normal problem skipped (B=2) and Fx prescribed
  (F=1), case 17 transient rolling from rest with Fx prescribed (T=2, TangCG), case 25 a shift
  of two very different materials (G 2e7 and 200) on a 251x1 strip with up to 30 outer
  iterations, and the cases that continue from the previous time instance: 11 (after 10),
  14-16 (transient rolling after 13) and 26 (after 25, the surface tilted).  The other cases
  use features outside this library (ConvexGS, bilinear loading,
  falling or variable friction, other materials, transient sequences, Fastsim).

* perfc_test/*.inp + perfc_test/get_times.ref_out -> perfc_cases.json
  the reference's performance inputs that this library solves (normal problems 1p-8p,
  1f-4f on 71x81 to 575x647 grids; shift problems 1s-8s), read with contact_gb300.inp
  (the geometry kept as its IBASE-2 table), with the published contact/slip counts,
  iteration counts and wall-clock seconds of the reference's 2016 performance run.

Usage: python tests/golden/make_golden.py [reference_root]
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def parse_test_table(path):
    lines = open(path).read().splitlines()
    hertz = []
    for ln in lines[:5]:
        m = re.search(r"a/b=\s*([\d.]+): rho=\s*([\d.Ee+-]+)\s*, cp=\s*([\d.Ee+-]+)", ln)
        hertz.append({"aob": float(m.group(1)), "rho": float(m.group(2)), "cp": float(m.group(3))})
    cases = []
    for ln in lines[5:]:
        vals = [t.split("=")[1].strip() for t in ln.split(",")]
        cases.append([float(vals[0]), float(vals[1]), float(vals[2]), float(vals[3])])
    return {"source": "testbank/test_table_mx11.ref_fx", "hertz": hertz, "cases": cases}


def parse_tractcurv(path, inp_path, ncase_max=30):
    # exact creepages of the first series from the input file
    cksi = [float(l.split()[1]) for l in open(inp_path) if "FN, CKSI, CETA, CPHI" in l][:ncase_max]
    text = open(path).read()
    blocks = re.split(r"\n Case\s+(\d+)\n", text)
    out = []
    for k in range(1, len(blocks), 2):
        icase = int(blocks[k])
        body = blocks[k + 1]
        if icase > ncase_max:
            break
        rec = {"case": icase}
        m = re.search(r"ItCG=\s*(\d+)", body)
        rec["itcg"] = int(m.group(1)) if m else None
        m = re.search(r"ItGS=\s*(\d+)", body)
        rec["itgs"] = int(m.group(1)) if m else None
        ln = body.splitlines()
        for i, s in enumerate(ln):
            if s.strip().startswith("FN") and "ELAST.EN." in s:
                v = ln[i + 1].split()
                rec.update(fn=float(v[0]), fx=float(v[1]), fy=float(v[2]), mz=float(v[3]),
                           elen=float(v[4]), frpow=float(v[5]))
            if s.strip().startswith("FN/G"):
                v = ln[i + 1].split()
                rec.update(fn_g=float(v[0]), fx_rel=float(v[1]), fy_rel=float(v[2]),
                           approach=float(v[3]), pmax=float(v[4]))
            if s.strip().startswith("NPOT") and "NCON" in s:
                v = ln[i + 1].split()
                rec.update(npot=int(v[0]), ncon=int(v[1]), nadh=int(v[2]), nslip=int(v[3]),
                           inorm=int(v[4]), itang=int(v[5]))
            if "FORM OF THE CONTACT" in s:
                rows = []
                j = i + 1
                while re.match(r"^\s+\d+\s+\S+$", ln[j]):
                    rows.append(ln[j].split()[1])
                    j += 1
                rec["picture"] = rows[::-1]     # row iy=1 first
        rec["cksi"] = cksi[icase - 1]
        out.append(rec)
    return {"source": "examples/tractcurv.ref_out", "series": 1, "cases": out}


def _results_block(body):
    """Printed results of one case: forces, approach, pmax, counts, picture."""
    rec = {}
    ln = body.splitlines()
    for i, s in enumerate(ln):
        if s.strip().startswith("FN") and "ELAST.EN." in s:
            v = ln[i + 1].split()
            rec.update(fn=float(v[0]), fx=float(v[1]), fy=float(v[2]), mz=float(v[3]), elen=float(v[4]))
        if s.strip().startswith("FN/G"):
            v = ln[i + 1].split()
            rec.update(approach=float(v[3]), pmax=float(v[4]))
        if s.strip().startswith("NPOT") and "NCON" in s:
            v = ln[i + 1].split()
            rec.update(npot=int(v[0]), ncon=int(v[1]), nadh=int(v[2]), nslip=int(v[3]))
            if len(v) >= 6 and "INORM" in s:
                rec.update(inorm=int(v[4]), itang=int(v[5]))
        if "FORM OF THE CONTACT" in s:
            rows = []
            j = i + 1
            while re.match(r"^\s+\d+\s+\S", ln[j]) and not ln[j].strip().startswith("1 2"):
                parts = ln[j].split()
                # a picture row: its row number, then one symbol per element (the column
                # numbers below the picture are digits)
                if not parts[0].isdigit() or len(parts) < 2 or any(t.isdigit() for t in parts[1:]):
                    break
                rows.append("".join(parts[1:]))
                j += 1
            rec["picture"] = rows[::-1]     # row iy=1 first
    return rec


def _nr_history(body):
    """The Newton-Raphson iterations on prescribed total forces (m_solvpt.f90:152-160, 336-347):
    per iteration [itnr, cksi, Fx/(mu Fn), ceta, Fy/(mu Fn), solver iterations]; ceta and Fy are
    None where only Fx is prescribed (F=1)."""
    num = r"(\S+)"
    rows = []
    for m in re.finditer(r"\n\s+(\d+), NR_F(x|y),\s+Cksi, Fxk:\s+" + num + r"\s+" + num +
                         r"(?:\s+It(?:CG|GS|GD):\s+(\d+))?(?:\n\s+Ceta, Fyk:\s+" + num + r"\s+" + num +
                         r"\s+It(?:CG|GS|GD):\s+(\d+))?", body):
        if m.group(2) == "x":
            rows.append([int(m.group(1)), float(m.group(3)), float(m.group(4)), None, None, int(m.group(5))])
        else:
            rows.append([int(m.group(1)), float(m.group(3)), float(m.group(4)), float(m.group(6)),
                         float(m.group(7)), int(m.group(8))])
    return rows


def _sensitivities(body):
    """The printed table of sensitivities: rows FN, FX, FY; columns d/dpen, d/dksi, d/deta,
    d/dphi (zero where not computed)."""
    ln = body.splitlines()
    for i, s in enumerate(ln):
        if s.strip().startswith("DF/DPEN"):
            return [[float(v) for v in ln[i + j].split()[1:5]] for j in (1, 2, 3)]
    return None


def _tang_final(rec, body):
    """Element counts and iterations of the case's last TANG solve (the last outer iteration
    where the normal and tangential problems are solved alternately)."""
    ms = list(re.finditer(r"Tang: final element division: A, S=\s*(\d+)\s+(\d+)\s+It(CG|GS)=\s*(\d+)", body))
    m = ms[-1] if ms else None
    if m:
        rec["tang_nadh"], rec["tang_nslip"] = int(m.group(1)), int(m.group(2))
        rec["tang_solver"], rec["tang_it"] = m.group(3), int(m.group(4))


def parse_cattaneo(path):
    text = open(path).read()
    blocks = re.split(r"\n Case\s+(\d+)\n", text)
    out = []
    for k in range(1, len(blocks), 2):
        icase = int(blocks[k])
        body = blocks[k + 1]
        rec = {"case": icase}
        m = re.search(r"Norm: final element division: C, E=\s*(\d+)\s+(\d+)\s+ItCG=\s*(\d+)", body)
        rec["norm_ncon"], rec["norm_itcg"] = int(m.group(1)), int(m.group(3))
        nr = _nr_history(body)
        if nr:
            rec["nr"] = nr
            rec["cksi"], rec["fx_rel_nr"] = nr[-1][1], nr[-1][2]
            rec["sens"] = _sensitivities(body)
        _tang_final(rec, body)
        rec.update(_results_block(body))
        out.append(rec)
    return {"source": "examples/cattaneo.ref_out", "cases": out}


def parse_catt_to_cart_case1(path):
    """Case 1 of examples/catt_to_cart.inp: the Cattaneo shift with Fx prescribed (F=1)."""
    text = open(path).read()
    blocks = re.split(r"\n Case\s+(\d+)\n", text)
    body = blocks[2]
    assert int(blocks[1]) == 1
    rec = {"case": 1}
    m = re.search(r"Norm: final element division: C, E=\s*(\d+)\s+(\d+)\s+ItCG=\s*(\d+)", body)
    rec["norm_ncon"], rec["norm_itcg"] = int(m.group(1)), int(m.group(3))
    rec["nr"] = _nr_history(body)
    rec["sens"] = _sensitivities(body)
    _tang_final(rec, body)
    rec.update(_results_block(body))
    m = re.search(r"FN/G\s+SHIFT X.*\n\s*(\S+)\s+(\S+)", body)
    rec["shift_x"] = float(m.group(2))
    return {"source": "examples/catt_to_cart.ref_out", "cases": [rec]}


def _table_after(ln, title, ncol):
    """Rows of the element table that follows a debug title (ix, iy, ii, then numbers)."""
    i = next(k for k, t in enumerate(ln) if t.strip() == title)
    rows = []
    for t in ln[i + 1:]:
        parts = [p for p in t.replace(",", " ").split()]
        if len(parts) == ncol and parts[0].isdigit():
            rows.append([float(p) for p in parts])
        elif rows:
            break
    return rows


def parse_carter2d(path):
    """examples/carter2d.inp: Carter's two-dimensional rolling problem (55x1 strip, SteadyGS),
    printed with element tables: the normal solution (approach to 8 digits, pn per element to
    4 decimals) and the tangential one after the slip-area update (element code, px to 4
    decimals, shift sx to 7 decimals)."""
    text = open(path).read()
    body = re.split(r"\n Case\s+(\d+)\n", text)[2]
    ln = body.splitlines()
    rec = {"case": 1}
    m = re.search(r"Norm: final element division: C, E=\s*(\d+)\s+(\d+)\s+ItCG=\s*(\d+)", body)
    rec["norm_ncon"], rec["norm_itcg"] = int(m.group(1)), int(m.group(3))
    _tang_final(rec, body)
    rec["pen8"] = float(re.search(r"Nmdbg: solution of NORM:\n pen =\s*(\S+)", body).group(1))
    norm = _table_after(ln, "Nmdbg: solution of NORM:", 9)
    rec["pn"] = [r[8] for r in norm]
    rec["norm_code"] = [int(r[7]) for r in norm]
    tang = _table_after(ln, "Nmdbg: after expanding slip-area:", 9)
    rec["tang_code"] = [int(r[3]) for r in tang]
    rec["tang_ii"] = [int(r[2]) for r in tang]
    rec["px"] = [r[4] for r in tang]
    rec["sx"] = [r[6] for r in tang]
    rec.update(_results_block(body))
    return {"source": "examples/carter2d.ref_out", "cases": [rec]}


def parse_testbank(path, wanted=(1, 4, 6, 7, 9, 10, 11, 13, 14, 15, 16, 17, 25, 26)):
    text = open(path).read()
    blocks = re.split(r"\n Case\s+(\d+)\n", text)
    out = []
    for k in range(1, len(blocks), 2):
        icase = int(blocks[k])
        if icase not in wanted:
            continue
        body = blocks[k + 1]
        rec = {"case": icase}
        ms = re.findall(r"Norm: final element division: C, E=\s*(\d+)\s+(\d+)\s+ItCG=\s*(\d+)", body)
        rec["norm_itcg"] = int(ms[-1][2]) if ms else 0          # last NORM; 0: skipped (B=2)
        _tang_final(rec, body)
        nr = _nr_history(body)
        if nr:
            rec["nr"] = nr
            rec["sens"] = _sensitivities(body)
        outer = re.findall(r"\d+, Panag/Out: \|Pk - Pk-1\|,  5 Eps \|Pk\| :\s*(\S+)\s+(\S+)", body)
        if outer:
            rec["outer"] = [[float(a), float(b)] for a, b in outer]
        rec.update(_results_block(body))
        out.append(rec)
    return {"source": "testbank/testbank.ref_out", "cases": out}


PERFC = ["norm_problm_1p", "norm_problm_2p", "norm_problm_4p", "norm_problm_8p", "norm_problm_1f",
         "norm_problm_2f", "norm_problm_4f", "tang_problm_1s", "tang_problm_2s", "tang_problm_4s",
         "tang_problm_8s"]


def parse_perfc(root):
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from contact_gb300 import inp
    times = {}
    for ln in open(os.path.join(root, "perfc_test", "get_times.ref_out")):
        m = re.match(r"(\w+): (ncon|nslp)=\s*(\d+), (ItCG|ItGS)=\s*(\d+), (?:tot|wall)\.(?:wall|tang)=\s*([\d.]+)", ln)
        if m:
            times[m.group(1)] = {m.group(2): int(m.group(3)), m.group(4).lower(): int(m.group(5)),
                                 "wall_s": float(m.group(6))}
    out = []
    for name in PERFC:
        cases = inp.read_inp(open(os.path.join(root, "perfc_test", name + ".inp")).read())
        c = {k: v for k, v in cases[0].items() if k != "h"}
        out.append({"name": name, "case": c, "reference": times[name]})
    return {"source": "perfc_test/*.inp, perfc_test/get_times.ref_out (2016-07-29, 1 thread)", "cases": out}


def parse_contact_nonhz(path):
    """testbank/contact_nonhz.ref_out, result element 1, first case: the call sequence of
    src/test_caddon.f90's element 1 printed by the library in CONTACT units."""
    text = open(path).read()
    body = re.split(r"\n Case\s+1 for contact problem\s+\d+ on result element\s+1\n", text)[1]
    body = re.split(r"\n Case\s+\d+ for contact problem", body)[0]
    rec = {"element": 1, "case": 1}
    m = re.search(r"Norm: final element division: C, E=\s*(\d+)\s+(\d+)\s+ItCG=\s*(\d+)", body)
    rec["norm_ncon"], rec["norm_itcg"] = int(m.group(1)), int(m.group(3))
    _tang_final(rec, body)
    rec.update(_results_block(body))
    return {"source": "testbank/contact_nonhz.ref_out", "units": "CONTACT (mm, N, forces on body 1)",
            "cases": [rec]}


SUBS_PICK = (0, 4, 8, 10, 12, 16, 20)      # x and y indices of the 21 x 21 block kept in the fixture


def parse_subsurf(root):
    """examples/subsurf.inp: one 1x1 mm element, G 1, nu 0.28, pn = 1; case 1 the pressure
    alone, case 2 with the traction px = 0.999 (Fx prescribed, the element in adhesion).
    From subsurf.ref_subs (written by case 2): the field at all 15 depths of block 1 and of a
    7x7 subgrid of block 2, as printed (the strings keep their printed precision); from
    subsurf.ref_out: the printed block summaries (maxima and their positions) of both
    cases."""
    rows = [ln.split() for ln in open(os.path.join(root, "examples", "subsurf.ref_subs"))
            if not ln.startswith("%")]
    heads = [i for i, r in enumerate(rows) if len(r) == 14 and r[3] == "0.000"]
    b1 = rows[heads[0] + 1:heads[1]]
    b2 = rows[heads[1] + 1:]
    n2 = 21
    keep2 = [r for k, r in enumerate(b2) if (k % n2) in SUBS_PICK and ((k // n2) % n2) in SUBS_PICK]
    text = open(os.path.join(root, "examples", "subsurf.ref_out")).read()
    solves = []
    for case_no, body in enumerate(re.split(r"\n Case\s+\d+\n", text)[1:], start=1):
        rec = {"case": case_no}
        m = re.search(r"Norm: final element division: C, E=\s*(\d+)\s+(\d+)\s+ItCG=\s*(\d+)", body)
        rec["norm_itcg"] = int(m.group(3))
        _tang_final(rec, body)
        nr = _nr_history(body)
        if nr:
            rec["nr"] = nr
            rec["sens"] = _sensitivities(body)
        rec.update(_results_block(body))
        rec.pop("picture", None)
        solves.append(rec)
    summaries = []
    for case_no, body in enumerate(re.split(r"\n Case\s+\d+\n", text)[1:], start=1):
        for nb, blk in re.findall(r"SUBSURFACE STRESSES BLOCK\s+(\d):\s*\n(.*?)\n\n", body + "\n\n", re.S):
            for ln in blk.strip().splitlines():
                m = re.match(r"\s*(ABSMAX|MAX|MIN)\s+(\w+)\s*=\s*(\S+)\s+AT \(X,Y,Z\) = \(\s*(\S+),\s*(\S+),\s*(\S+)\)",
                             ln)
                if m:
                    summaries.append({"case": case_no, "block": int(nb), "kind": m.group(1), "quantity": m.group(2),
                                      "value": float(m.group(3)), "at": [float(m.group(k)) for k in (4, 5, 6)]})
    return {"source": "examples/subsurf.ref_subs, examples/subsurf.ref_out",
            "columns": ["X", "Y", "Z", "UX", "UY", "UZ", "SIGHYD", "SIGVM", "SIGXX", "SIGXY", "SIGXZ", "SIGYY",
                        "SIGYZ", "SIGZZ"],
            "gg": 1.0, "poiss": 0.28,
            "block1": b1, "block2_subgrid": keep2, "block2_pick": list(SUBS_PICK),
            "block2_x": [float(r[0]) for r in b2[:n2]], "block2_y": [float(b2[k * n2][1]) for k in range(n2)],
            "block2_z": [float(b2[k * n2 * n2][2]) for k in range(len(b2) // (n2 * n2))], "summaries": summaries,
            "solves": solves}


def parse_bentall(root):
    """examples/bentall.inp: steady rolling of two different materials on a 216x1 strip at chi =
    180 deg, Fx prescribed, the normal and tangential problems coupled: the reader's six cases
    (replayed in order, case 2 starting from case 1's solution) and the printed results of
    cases 2-6 (case 1 prints none): every Newton-Raphson row over all outer iterations, the
    last solve's counts and iterations, the number of outer iterations, forces, energy,
    approach, pmax, creepage, sensitivities and the picture."""
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from contact_gb300 import inp
    cases = inp.read_inp(open(os.path.join(root, "examples", "bentall.inp")).read())
    text = open(os.path.join(root, "examples", "bentall.ref_out")).read()
    blocks = re.split(r"\n Case\s+(\d+)\n", text)
    out = []
    for k in range(1, len(blocks), 2):
        body = blocks[k + 1]
        if "TOTAL FORCES" not in body:
            continue
        rec = {"case": int(blocks[k])}
        ms = re.findall(r"Norm: final element division: C, E=\s*(\d+)\s+(\d+)\s+ItCG=\s*(\d+)", body)
        rec["norm_itcg"] = int(ms[-1][2])
        _tang_final(rec, body)
        rec["nr"] = _nr_history(body)
        rec["sens"] = _sensitivities(body)
        m = re.search(r"FN/G\s+CREEP X.*\n\s*(\S+)\s+(\S+)", body)
        rec["cksi"] = float(m.group(2))
        rec.update(_results_block(body))
        out.append(rec)
    return {"source": "examples/bentall.inp, examples/bentall.ref_out", "inputs": cases, "cases": out}


def parse_catt_to_cart(root):
    """examples/catt_to_cart.inp, all 171 cases: three sequences from a Cattaneo shift into
    rolling (transient rolling, T=2, on a fixed 34x33 grid; shifts on a world-fixed 90x33 grid;
    shifts on a 34x33 grid that moves one element per step), each case continuing from the
    previous time instance (P=0) with Fx prescribed: the reader's cases, to be replayed in
    order, and per case the printed Newton-Raphson rows, and the counts where printed."""
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from contact_gb300 import inp
    cases = inp.read_inp(open(os.path.join(root, "examples", "catt_to_cart.inp")).read())
    for c in cases:
        for k, v in list(c.items()):
            if hasattr(v, "tolist"):
                c[k] = v.tolist()
    text = open(os.path.join(root, "examples", "catt_to_cart.ref_out")).read()
    blocks = re.split(r"\n Case\s+(\d+)\n", text)
    out = []
    for k in range(1, len(blocks), 2):
        body = blocks[k + 1]
        rec = {"case": int(blocks[k]), "nr": _nr_history(body)}
        res = _results_block(body)
        for key in ("ncon", "nadh", "nslip", "fn", "fx", "approach", "pmax"):
            if key in res:
                rec[key] = res[key]
        out.append(rec)
    return {"source": "examples/catt_to_cart.inp, examples/catt_to_cart.ref_out", "inputs": cases, "cases": out}


def parse_spence35(root):
    """examples/spence35.inp, all 35 cases: Spence's problem, a sphere of one material pressed
    into and lifted off a half-space of another (the normal and tangential problems coupled)
    in 35 load steps, each continuing from the previous one (P=0), with subsurface stresses
    along one grid row: the reader's cases and per case the printed outer iterations, totals
    and counts where printed, and the printed subsurface maxima of cases 6, 18 and 35."""
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from contact_gb300 import inp
    cases = inp.read_inp(open(os.path.join(root, "examples", "spence35.inp")).read())
    text = open(os.path.join(root, "examples", "spence35.ref_out")).read()
    blocks = re.split(r"\n Case\s+(\d+)\n", text)
    out = []
    for k in range(1, len(blocks), 2):
        body = blocks[k + 1]
        rec = {"case": int(blocks[k])}
        rec["outer"] = [[float(a), float(b)] for a, b in
                        re.findall(r"Panag/Out: \|Pk - Pk-1\|,  5 Eps \|Pk\| :\s*(\S+)\s+(\S+)", body)]
        res = _results_block(body)
        res.pop("picture", None)
        rec.update(res)
        subs = []
        for nb, blk in re.findall(r"SUBSURFACE STRESSES BLOCK\s+(\d):\s*\n(.*?)\n\n", body + "\n\n", re.S):
            for ln in blk.strip().splitlines():
                m = re.match(r"\s*(ABSMAX|MAX|MIN)\s+(\w+)\s*=\s*(\S+)\s+AT \(X,Y,Z\) = \(\s*(\S+),\s*(\S+),\s*(\S+)\)",
                             ln)
                if m:
                    subs.append({"block": int(nb), "kind": m.group(1), "quantity": m.group(2),
                                 "value": float(m.group(3)), "at": [float(m.group(j)) for j in (4, 5, 6)]})
        if subs:
            rec["subs"] = subs
        out.append(rec)
    return {"source": "examples/spence35.inp, examples/spence35.ref_out", "inputs": cases, "cases": out}


def parse_veldep_fric(root):
    """Case 1 of examples/veldep_fric.inp: steady rolling on a 92x1 strip (ConvexGS) with an
    exponential falling friction law (L=4): the reader's case and the printed iterations on
    the slip velocity (adhesion and slip counts, the change of the slip velocities and its
    tolerance), the ConvexGS sweeps, counts and totals."""
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from contact_gb300 import inp
    case = inp.read_inp(open(os.path.join(root, "examples", "veldep_fric.inp")).read())[0]
    case = {k: (v.tolist() if hasattr(v, "tolist") else v) for k, v in case.items()}
    body = re.split(r"\n Case\s+\d+\n", open(os.path.join(root, "examples", "veldep_fric.ref_out")).read())[1]
    rec = {"slp": [[int(a), int(b), float(c), float(d)] for a, b, c, d in
                   re.findall(r"Vel-dep: A, S=\s*(\d+)\s+(\d+), \|Sk-Sk-1\|, \.001 \|Sk\| :\s*(\S+)\s+(\S+)", body)]}
    m = re.search(r"Norm: final element division: C, E=\s*(\d+)\s+(\d+)\s+ItCG=\s*(\d+)", body)
    rec["norm_ncon"], rec["norm_itcg"] = int(m.group(1)), int(m.group(3))
    _tang_final(rec, body)
    res = _results_block(body)
    res.pop("picture", None)
    rec.update(res)
    return {"source": "examples/veldep_fric.inp, examples/veldep_fric.ref_out (case 1)", "input": case,
            "result": rec}


def parse_tractcurv_series2(root):
    """Cases 31-60 of examples/tractcurv.inp, the series with an interfacial layer (M=4, TAU_C0 0)
    and exponential falling friction with a friction memory: the reader's cases and per case
    the printed slip-velocity iterations (the change of the slip velocities and its tolerance),
    the NormCG and SteadyGS iterations, counts, totals and the element-division picture."""
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from contact_gb300 import inp
    cases = inp.read_inp(open(os.path.join(root, "examples", "tractcurv.inp")).read())[30:60]
    cases = [{k: (v.tolist() if hasattr(v, "tolist") else v) for k, v in c.items()} for c in cases]
    blocks = re.split(r"\n Case\s+(\d+)\n", open(os.path.join(root, "examples", "tractcurv.ref_out")).read())
    out = []
    for k in range(1, len(blocks), 2):
        icase = int(blocks[k])
        if not 31 <= icase <= 60:
            continue
        body = blocks[k + 1]
        rec = {"case": icase,
               "slp": [[float(c), float(d)] for c, d in
                       re.findall(r"Vel-dep: \|Sk-Sk-1\|, \.001 \|Sk\| :\s*(\S+)\s+(\S+)", body)]}
        ms = re.findall(r"Norm: final element division: C, E=\s*(\d+)\s+(\d+)\s+ItCG=\s*(\d+)", body)
        rec["norm_itcg"] = int(ms[-1][2])
        _tang_final(rec, body)
        rec.update(_results_block(body))
        out.append(rec)
    return {"source": "examples/tractcurv.inp, examples/tractcurv.ref_out (cases 31-60)", "inputs": cases,
            "cases": out}


def parse_testbank_case3(path):
    """Case 3 of testbank/testbank.inp: the normal problem of two bodies (G 200 and 1) on a 3x3
    Hertzian grid with one element in contact, and the subsurface field at six points in both
    bodies: per point x, y, z, the three displacements, the stress tensor row by row, SigHyd and
    SigVM as printed (strings), and the block's printed maxima."""
    body = re.split(r"\n Case\s+(\d+)\n", open(path).read())
    body = body[body.index("3") + 1]
    s = r"\s*(\S+?)\s*"
    pts = []
    for m in re.finditer(r"Position \(X,Y,Z\):" + s * 3 + r"\n.*\n" +
                         "".join(r"\s*%d%s;%s%s%s\n" % (i, s, s, s, s) for i in (1, 2, 3)) +
                         r"\s*SigHyd =" + s + r", SigVM =" + s + r"\n", body):
        g = m.groups()
        pts.append(list(g[0:3]) + [g[3], g[7], g[11]] + list(g[4:7]) + list(g[8:11]) + list(g[12:15]) + list(g[15:17]))
    summ = []
    for ln in body.splitlines():
        m = re.match(r"\s*(ABSMAX|MAX|MIN)\s+(\w+)\s*=\s*(\S+)\s+AT \(X,Y,Z\) = \(\s*(\S+),\s*(\S+),\s*(\S+)\)", ln)
        if m:
            summ.append({"kind": m.group(1), "quantity": m.group(2).lower(), "value": float(m.group(3)),
                         "at": [float(m.group(k)) for k in (4, 5, 6)]})
    res = _results_block(body)
    return {"source": "testbank/testbank.ref_out (case 3)", "points": pts, "summaries": summ,
            "approach": res["approach"], "pmax": res["pmax"], "fn": res["fn"],
            "norm_itcg": int(re.search(r"ItCG=\s*(\d+)", body).group(1))}


def parse_veldep_sequence(root):
    """All 53 cases of examples/veldep_fric.inp, to be replayed in order: the reader's cases
    and per printed case its iterations on the slip velocity (adhesion and slip counts, the
    change of the slip velocities and its tolerance), the last tangential solve's iterations,
    counts and totals where printed."""
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from contact_gb300 import inp
    cases = inp.read_inp(open(os.path.join(root, "examples", "veldep_fric.inp")).read())
    cases = [{k: (v.tolist() if hasattr(v, "tolist") else v) for k, v in c.items()} for c in cases]
    blocks = re.split(r"\n Case\s+(\d+)\n", open(os.path.join(root, "examples", "veldep_fric.ref_out")).read())
    out = []
    for k in range(1, len(blocks), 2):
        body = blocks[k + 1]
        rec = {"case": int(blocks[k]),
               "slp": [[int(a), int(b), float(c), float(d)] for a, b, c, d in
                       re.findall(r"Vel-dep: A, S=\s*(\d+)\s+(\d+), \|Sk-Sk-1\|, \.001 \|Sk\| :\s*(\S+)\s+(\S+)", body)]}
        _tang_final(rec, body)
        res = _results_block(body)
        res.pop("picture", None)
        rec.update(res)
        out.append(rec)
    return {"source": "examples/veldep_fric.inp, examples/veldep_fric.ref_out", "inputs": cases, "cases": out}


def parse_test_caddon(path):
    text = open(path).read()
    block = text.split("...start processing of Result Element")[1]     # element 1, first solve
    num = r"([-+]?[\d.]+(?:[EeDd][-+]?\d+)?)"
    rec = {}
    m = re.search(r"Dx=\s*" + num + r", Dy=\s*" + num, block)
    rec["dx_m"], rec["dy_m"] = float(m.group(1)), float(m.group(2))
    rec["pen_m"] = float(re.search(r"Pen=\s*" + num, block).group(1))
    m = re.search(r"Tn=\s*" + num + r", Fx=\s*" + num + r", Fy=\s*" + num + r" \[N\], Mz=\s*" + num, block)
    rec["tn"], rec["fx"], rec["fy"], rec["mz_nm"] = (float(m.group(k)) for k in range(1, 5))
    m = re.search(r"Mx=\s*(\d+), My=\s*(\d+)", block)
    rec["mx"], rec["my"] = int(m.group(1)), int(m.group(2))
    m = re.search(r"C=\s*" + num + r" \[m2\], H=\s*" + num + r" \[m2\], S=\s*" + num, block)
    rec["carea_m2"], rec["harea_m2"], rec["sarea_m2"] = (float(m.group(k)) for k in range(1, 4))
    m = re.search(r"Pnmax=\s*" + num + r", Ptmax=\s*" + num, block)
    rec["pnmax_mpa"], rec["ptmax_mpa"] = float(m.group(1)), float(m.group(2))
    for key in ("Pn", "Px", "Py"):
        m = re.search(key + r"\(\s*(\d+),\s*(\d+)\)=\s*" + num, block)
        rec[key.lower() + "_max"] = [int(m.group(1)), int(m.group(2)), float(m.group(3))]
    return {"source": "testbank/test_caddon.ref_out", "element": 1, "units": "SPCK (m, N, forces on body 2)",
            "result": rec}


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    tt = parse_test_table(os.path.join(root, "testbank", "test_table_mx11.ref_fx"))
    with open(os.path.join(HERE, "test_table_mx11.json"), "w") as f:
        json.dump(tt, f, separators=(",", ":"))
    tc = parse_tractcurv(os.path.join(root, "examples", "tractcurv.ref_out"),
                         os.path.join(root, "examples", "tractcurv.inp"))
    with open(os.path.join(HERE, "tractcurv_series1.json"), "w") as f:
        json.dump(tc, f, indent=0)
    ca = parse_cattaneo(os.path.join(root, "examples", "cattaneo.ref_out"))
    with open(os.path.join(HERE, "cattaneo.json"), "w") as f:
        json.dump(ca, f, indent=0)
    cs = parse_catt_to_cart(root)
    with open(os.path.join(HERE, "catt_to_cart_sequence.json"), "w") as f:
        json.dump(cs, f, separators=(",", ":"))
    cc = parse_catt_to_cart_case1(os.path.join(root, "examples", "catt_to_cart.ref_out"))
    with open(os.path.join(HERE, "catt_to_cart_case1.json"), "w") as f:
        json.dump(cc, f, indent=0)
    c2 = parse_carter2d(os.path.join(root, "examples", "carter2d.ref_out"))
    with open(os.path.join(HERE, "carter2d.json"), "w") as f:
        json.dump(c2, f, indent=0)
    cn = parse_contact_nonhz(os.path.join(root, "testbank", "contact_nonhz.ref_out"))
    with open(os.path.join(HERE, "contact_nonhz_re1.json"), "w") as f:
        json.dump(cn, f, indent=0)
    ss = parse_subsurf(root)
    with open(os.path.join(HERE, "subsurf.json"), "w") as f:
        json.dump(ss, f, separators=(",", ":"))
    bt = parse_bentall(root)
    with open(os.path.join(HERE, "bentall.json"), "w") as f:
        json.dump(bt, f, indent=0)
    sp = parse_spence35(root)
    with open(os.path.join(HERE, "spence35.json"), "w") as f:
        json.dump(sp, f, separators=(",", ":"))
    vf = parse_veldep_fric(root)
    with open(os.path.join(HERE, "veldep_fric_case1.json"), "w") as f:
        json.dump(vf, f, indent=0)
    with open(os.path.join(HERE, "testbank_case3_subs.json"), "w") as f:
        json.dump(parse_testbank_case3(os.path.join(root, "testbank", "testbank.ref_out")), f, indent=0)
    t2 = parse_tractcurv_series2(root)
    with open(os.path.join(HERE, "tractcurv_series2.json"), "w") as f:
        json.dump(t2, f, separators=(",", ":"))
    vs = parse_veldep_sequence(root)
    with open(os.path.join(HERE, "veldep_fric_sequence.json"), "w") as f:
        json.dump(vs, f, separators=(",", ":"))
    tcd = parse_test_caddon(os.path.join(root, "testbank", "test_caddon.ref_out"))
    with open(os.path.join(HERE, "test_caddon_re1.json"), "w") as f:
        json.dump(tcd, f, indent=0)
    tb = parse_testbank(os.path.join(root, "testbank", "testbank.ref_out"))
    with open(os.path.join(HERE, "testbank_cases.json"), "w") as f:
        json.dump(tb, f, indent=0)
    pf = parse_perfc(root)
    with open(os.path.join(HERE, "perfc_cases.json"), "w") as f:
        json.dump(pf, f, separators=(",", ":"))
    print("test_table cases:", len(tt["cases"]), " tractcurv cases:", len(tc["cases"]),
          " cattaneo cases:", len(ca["cases"]), " test_caddon element 1:", tcd["result"]["tn"])


if __name__ == "__main__":
    main()
