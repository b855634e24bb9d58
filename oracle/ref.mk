# Builds the BlochLib reference's powder-FID path (scratch copy made by build_ref.sh)
# plus oracle/ref_harness.cc.  Test infrastructure only; outputs go to oracle/_ref/.
#   make -f ref.mk QL=float  BIN=_ref/ref_fid    OBJ=_ref/obj_f32
#   make -f ref.mk QL=double BIN=_ref/ref_fid64  OBJ=_ref/obj_f64
SRC ?= _ref/src
OBJ ?= _ref/obj_f32
QL ?= float
BIN ?= _ref/ref_fid
CXX ?= g++
OPT ?= -O2
RED ?= _ref/mmmqmas
CXXFLAGS = -std=gnu++98 -fpermissive -w $(OPT) -include ref_prelude.h -DBL_QL_REAL=$(QL) -I$(SRC) -I$(RED)

TUS = version.cc container/complex.cc container/range.cc \
  utils/blassert.cc utils/params.cc utils/endians.cc utils/matlab5.cc utils/utils.cc \
  utils/constants.cc utils/random.cc utils/plotter.cc utils/parser.cc utils/scriptparse.cc \
  mpi/mpi_config.cc mpi/mpi_tools.cc mpi/mpi_controller.cc \
  container/matrix/matmatmul.cc container/matrix/matdiagonalize.cc container/matrix/matexp.cc \
  container/matrix/mdmd_a1bc_md_cm.cc container/matrix/mdmd_acbc_md_cm.cc \
  container/matrix/mdmdt_a1bc_md_cm.cc container/matrix/mdmdt_acbc_md_cm.cc \
  container/matrix/mdtmd_a1bc_md_cm.cc container/matrix/mdtmd_acbc_md_cm.cc \
  container/matrix/mdtmdt_a1bc_md_cm.cc container/matrix/mdtmdt_acbc_md_cm.cc \
  bloch/Isotope.cc \
  QMspins/multispinop.cc QMspins/singlespinop.cc QMspins/spinsys.cc QMspins/spinsyspars.cc \
  QMspins/space_ten.cc QMspins/spin_ten.cc QMspins/sys.cc QMspins/j.cc QMspins/csa.cc \
  QMspins/dip.cc QMspins/qua.cc QMspins/driver/powder.cc QMspins/driver/ham_gen.cc

OBJS = $(patsubst %.cc,$(OBJ)/%.o,$(TUS)) $(OBJ)/propreduce.o $(OBJ)/ref_harness.o

$(BIN): $(OBJS)
	$(CXX) -o $@ $(OBJS) -lm

$(OBJ)/ref_harness.o: ref_harness.cc $(RED)/propreduce.h
	@mkdir -p $(dir $@)
	$(CXX) $(CXXFLAGS) -c $< -o $@

$(OBJ)/propreduce.o: $(RED)/propreduce.cc $(RED)/propreduce.h
	@mkdir -p $(dir $@)
	$(CXX) $(CXXFLAGS) -c $< -o $@

$(OBJ)/%.o: $(SRC)/%.cc
	@mkdir -p $(dir $@)
	$(CXX) $(CXXFLAGS) -c $< -o $@
