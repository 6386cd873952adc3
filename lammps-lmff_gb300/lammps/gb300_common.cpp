/* ----------------------------------------------------------------------
   Parts the GB300 pair styles share -- see gb300_common.h
------------------------------------------------------------------------- */

#include "gb300_common.h"

#include <string>

#include "atom.h"
#include "comm.h"
#include "domain.h"
#include "error.h"
#include "force.h"
#include "lammps.h"
#include "neighbor.h"
#include "pair.h"

using namespace LAMMPS_NS;

namespace {

// the other gb300 style of the same hybrid/overlay (Force::pair_match looks through the
// sub-styles; a second instance of a style makes the match ambiguous and gives NULL)
Pair *find_partner(LAMMPS *lmp, Pair *self, int slot, GB300Style **pc)
{
  static const char *inter[] = {"^ilp/graphene/hbn", "^kolmogorov/crespi/full"};
  static const char *ters[] = {"^tersoff"};
  const char **pat = slot == 0 ? inter : ters;
  int npat = slot == 0 ? 2 : 1;
  for (int k = 0; k < npat; k++) {
    Pair *p = lmp->force->pair_match(pat[k],0);
    if (!p || p == self) continue;
    GB300Style *g = dynamic_cast<GB300Style *>(p);
    if (g) {
      *pc = g;
      return p;
    }
  }
  *pc = NULL;
  return NULL;
}

}  // namespace

void gb300::setup(LAMMPS *lmp, Pair *self, GB300Style *me, int slot, const char *name)
{
  if (me->set_by_partner) {       // the partner's init_style made the shared engine
    me->set_by_partner = false;
    return;
  }
  GB300Style *pc = NULL;
  Pair *partner = find_partner(lmp,self,slot,&pc);
  lmff_lammps::StyleParams sp;
  me->fill_params(sp);
  if (pc) pc->fill_params(sp);
  std::string err;
  std::shared_ptr<lmff_lammps::Shared> s = std::make_shared<lmff_lammps::Shared>();
  if (s->ad.create(sp,lmff_lammps::device_from_env(),lmff_lammps::precision_from_env(),err) != LMFF_OK)
    lmp->error->all(FLERR,(std::string(name) + ": " + err).c_str());
  me->gb = s;
  me->partner = partner;
  if (pc) {
    pc->gb = s;
    pc->partner = self;
    pc->set_by_partner = true;
  }
}

void gb300::compute(LAMMPS *lmp, Pair *self, GB300Style *me, int slot, int eflag, int vflag, int eflag_atom,
                    int vflag_atom, const char *name, lmff_lammps::StyleOut &out)
{
  Atom *atom = lmp->atom;
  Domain *domain = lmp->domain;
  if (!me->gb) lmp->error->all(FLERR,(std::string(name) + ": engine not set up").c_str());

  // one MPI rank with an orthogonal box: the periodic form (owned atoms + box); a domain
  // decomposition or a triclinic box: the subdomain form (owned + ghost atoms, the
  // ghosts LAMMPS made carrying the periodic images)
  const bool sub = lmp->comm->nprocs > 1 || domain->triclinic || lmff_lammps::subdomain_from_env();
  const int nlocal = atom->nlocal;
  const int nall = nlocal + atom->nghost;
  const int n = sub ? nall : nlocal;
  const int periodic[3] = {domain->xperiodic, domain->yperiodic, domain->zperiodic};
  const bool big = sizeof(tagint) == 8;
  const tagint *mol = atom->molecule_flag ? atom->molecule : NULL;
  const bool partner_computes = me->partner && me->partner->compute_flag;
  std::string err;
  int rc = me->gb->evaluate(slot, partner_computes, nlocal, nall, sub, n ? &atom->x[0][0] : NULL, atom->type,
                            big ? NULL : (const int32_t *) mol, big ? (const int64_t *) mol : NULL,
                            big ? NULL : (const int32_t *) atom->tag, big ? (const int64_t *) atom->tag : NULL,
                            lmp->neighbor->ago == 0, domain->boxlo, domain->boxhi, periodic,
                            n ? &atom->f[0][0] : NULL, eflag_atom ? self->eatom : NULL,
                            (vflag_atom && n) ? &self->vatom[0][0] : NULL, eflag, vflag, out, err);
  if (rc != LMFF_OK) lmp->error->one(FLERR,(std::string(name) + ": " + err).c_str());
}
