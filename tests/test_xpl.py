"""XPL solver configuration (plask_gb300.xpl) applied to the drop-in solver objects, on the
CPU: the tags and attributes of ThermalFem3DSolver::loadConfiguration
(solvers/thermal/static/therm3d.cpp:40-69), fem_solver.hpp:38-106 and 164-178,
DynamicThermalFem3DSolver (femT3d.cpp:46-70), DynamicThermalFem2DSolver (femT2d.cpp:46-70)
and the Shockley solver (electr3d.cpp:41-87,
beta.cpp:26-62)."""
import numpy as np
import pytest

from plask_gb300 import electrical as EL
from plask_gb300 import thermal as TH
from plask_gb300 import thermal2d as T2
from plask_gb300 import xpl


def test_static3d_configuration():
    mesh = TH.RectangularMesh3D(np.linspace(0, 1, 3), np.linspace(0, 1, 3), np.linspace(0, 1, 4))
    sv = TH.Static3D("therm")
    xpl.configure(sv, """
      <thermal solver="Static3D" name="therm">
        <mesh ref="grid" empty-elements="include"/>
        <loop inittemp="290" maxerr="0.01"/>
        <matrix algorithm="iterative">
          <iterative maxit="2000" maxerr="1e-8" noconv="error" nfact="20" preconditioner="ic" nsave="7"/>
        </matrix>
        <temperature>
          <condition place="bottom" value="300" placename="floor"/>
        </temperature>
        <heatflux><condition placeref="floor" value="-1e3"/></heatflux>
        <convection><condition place="top" coeff="10" ambient="300"/></convection>
        <radiation><condition><place side="front"/></condition></radiation>
      </thermal>""".replace('<radiation><condition><place side="front"/></condition></radiation>',
                            '<radiation><condition emissivity="0.8" ambient="280"><place side="front"/></condition></radiation>'),
                  meshes={"grid": mesh})
    assert sv.mesh is mesh and sv.empty_elements == "include"
    assert sv.inittemp == 290.0 and sv.maxerr == 0.01
    assert sv.algorithm == "iterative"
    it = sv.iterative
    assert (it.maxit, it.maxerr, it.noconv, it.nfact, it.preconditioner, it.ns1) == (2000, 1e-8, "error", 20, "ic", 7)
    assert len(sv.temperature_boundary) == 1 and sv.temperature_boundary[0][1] == (300.0,)
    place, vals = sv.heatflux_boundary[0]
    assert vals == (-1e3,) and np.array_equal(place.mask(mesh), TH.RectangularMesh3D.Bottom().mask(mesh))
    assert sv.convection_boundary[0][1] == (10.0, 300.0)
    assert sv.radiation_boundary[0][1] == (0.8, 280.0)
    assert np.array_equal(sv.radiation_boundary[0][0].mask(mesh), TH.RectangularMesh3D.Front().mask(mesh))


def test_static2d_sides_and_errors():
    sv = T2.StaticCyl()
    xpl.configure(sv, '<thermal><temperature><condition place="right" value="310"/></temperature></thermal>')
    assert sv.temperature_boundary[0][1] == (310.0,)
    with pytest.raises(ValueError):
        xpl.configure(T2.Static2D(), '<thermal><temperature><condition place="front" value="1"/></temperature></thermal>')
    with pytest.raises(ValueError):
        xpl.configure(TH.Static3D(), '<thermal><temperature><condition value="1"><place object="mesa" side="top"/>'
                                     '</condition></temperature></thermal>')
    with pytest.raises(ValueError):
        xpl.configure(TH.Static3D(), '<thermal><matrix algorithm="lu"/></thermal>')


def test_dynamic3d_configuration():
    sv = TH.Dynamic3D()
    xpl.configure(sv, """<thermal solver="Dynamic3D">
        <loop inittemp="295" timestep="0.05" rebuildfreq="4" logfreq="10"/>
        <matrix methodparam="1.0" lumping="false" algorithm="cholesky"/>
        <temperature><condition place="bottom" value="300"/></temperature></thermal>""")
    assert (sv.inittemp, sv.timestep, sv.rebuildfreq, sv.logfreq) == (295.0, 0.05, 4, 10)
    assert sv.methodparam == 1.0 and sv.lumping is False and sv.algorithm == "cholesky"
    with pytest.raises(ValueError):
        xpl.configure(TH.Dynamic3D(), '<thermal><convection><condition place="top" coeff="1" ambient="300"/>'
                                      '</convection></thermal>')


@pytest.mark.parametrize("cls", [T2.Dynamic2D, T2.DynamicCyl])
def test_dynamic2d_configuration(cls):
    """DynamicThermalFem2DSolver::loadConfiguration (femT2d.cpp:46-70)."""
    sv = cls()
    xpl.configure(sv, """<thermal>
        <loop inittemp="310" timestep="0.5" rebuildfreq="2" logfreq="7"/>
        <matrix methodparam="0.75" lumping="no"/>
        <temperature><condition place="left" value="320"/></temperature></thermal>""")
    assert (sv.inittemp, sv.timestep, sv.rebuildfreq, sv.logfreq) == (310.0, 0.5, 2, 7)
    assert sv.methodparam == 0.75 and sv.lumping is False
    assert sv.temperature_boundary[0][1] == (320.0,)
    with pytest.raises(ValueError):
        xpl.configure(cls(), '<thermal><radiation><condition place="top" emissivity="0.5" ambient="300"/>'
                             '</radiation></thermal>')
    with pytest.raises(ValueError):
        xpl.configure(cls(), '<thermal><loop maxerr="0.1"/></thermal>')


def test_shockley3d_configuration():
    sv = EL.Shockley3D("el")
    xpl.configure(sv, """<electrical solver="Shockley3D">
        <voltage><condition place="top" value="1.5"/><condition place="bottom" value="0"/></voltage>
        <loop start-cond="0.1,2.5" convergence="stable" maxerr="0.1"/>
        <contacts pcond="7" ncond="70"/>
        <junction js="2" beta="19" beta1="17" js1="1.5"/>
      </electrical>""")
    assert len(sv.voltage_boundary) == 2 and sv.voltage_boundary[0][1] == (1.5,)
    assert sv.start_cond == (0.1, 2.5) and sv.convergence == "stable" and sv.maxerr == 0.1
    assert (sv.pcond, sv.ncond) == (7.0, 70.0)
    assert sv.js == 2.0 and sv.beta == 19.0 and sv.beta1 == 17.0 and sv.js1 == 1.5
    xpl.configure(sv, '<electrical><loop start-cond="3"/></electrical>')
    assert sv.start_cond == (0.1, 3.0)


def test_thermoelectric3d_configuration():
    """ThermoElectric._parse_xpl (solvers/meta/shockley/thermoelectric.py:131-172)."""
    te = EL.ThermoElectric3D()
    tmesh, emesh = object(), object()
    xpl.configure(te, """<thermoelectric>
        <mesh thermal="tm" electrical="em" empty-elements="include"/>
        <junction beta0="19" js0="1.5" pnjcond="0.3"/>
        <contacts pcond="7" ncond="8"/>
        <loop tfreq="4" inittemp="295" maxterr="0.1" maxcerr="0.2"/>
        <tmatrix algorithm="iterative"><iterative maxit="500"/></tmatrix>
        <ematrix algorithm="cholesky"/>
        <temperature><condition place="bottom" value="300"/></temperature>
        <convection><condition place="top" coeff="10" ambient="300"/></convection>
        <voltage><condition place="top" value="2"/><condition place="bottom" value="0"/></voltage>
        </thermoelectric>""", meshes={"tm": tmesh, "em": emesh})
    assert te.thermal.mesh is tmesh and te.electrical.mesh is emesh
    assert te.electrical.empty_elements == "include"
    assert (te.electrical.beta0, te.electrical.js0) == (19.0, 1.5)
    assert tuple(te.electrical.start_cond) == (0.0, 0.3)  # pnjcond sets the junction's start conductivity
    assert (te.electrical.pcond, te.electrical.ncond) == (7.0, 8.0)
    assert (te.tfreq, te.thermal.inittemp, te.thermal.maxerr, te.electrical.maxerr) == (4, 295.0, 0.1, 0.2)
    assert te.thermal.algorithm == "iterative" and te.thermal.iterative.maxit == 500
    assert te.electrical.algorithm == "cholesky"
    assert len(te.thermal.temperature_boundary) == 1 and len(te.thermal.convection_boundary) == 1
    assert [v for _, v in te.electrical.voltage_boundary] == [(2.0,), (0.0,)]
    with pytest.raises(ValueError):
        xpl.configure(EL.ThermoElectric3D(), "<thermoelectric><optical/></thermoelectric>")
