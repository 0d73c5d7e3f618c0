// compat_containers.cpp -- the hpg-libs container and alignment functions the
// alignment-list layer calls, for processes that do not link hpg-libs.
//
// A caller built against hpg-libs resolves these names to its own libhpg
// (loaded before this library, so the dynamic linker binds every call here,
// including this library's own, to libhpg's definitions); only a process
// without hpg-libs (tests, ctypes callers) runs these.  Layout and behaviour
// follow c/src/containers/array_list.{h,c} (array_list_t, growth by the
// realloc factor, the flag word, an optional lock),
// c/src/containers/linked_list.{h,c} (linked_list_t: doubly linked items,
// insert = at the head, insert_last = at the tail) and
// c/src/bioformats/bam/alignment.c:7-10,253-264 (zeroed allocation, free of
// the owned strings).
#include <pthread.h>

#include <cstdlib>
#include <cstring>

#include "hpg_bwt_api.h"

namespace {

void lock(array_list_t* l) {
  if (l->mode == COLLECTION_MODE_SYNCHRONIZED) pthread_mutex_lock(&l->lock);
}

void unlock(array_list_t* l) {
  if (l->mode == COLLECTION_MODE_SYNCHRONIZED) pthread_mutex_unlock(&l->lock);
}

bool grow(array_list_t* l) {
  size_t cap = (size_t)((double)l->capacity * (l->realloc_factor > 1.0f ? l->realloc_factor : 1.5f));
  if (cap < l->capacity + 4) cap = l->capacity + 4;
  void** items = static_cast<void**>(std::realloc(l->items, cap * sizeof(void*)));
  if (!items) return false;
  l->items = items;
  l->capacity = cap;
  return true;
}

}  // namespace

extern "C" {

array_list_t* array_list_new(size_t initial_capacity, float realloc_factor, int SYNC_MODE) {
  array_list_t* l = static_cast<array_list_t*>(std::calloc(1, sizeof(array_list_t)));
  if (!l) return nullptr;
  l->capacity = initial_capacity;
  l->realloc_factor = realloc_factor;
  l->mode = SYNC_MODE;
  l->items = static_cast<void**>(std::malloc((initial_capacity ? initial_capacity : 1) * sizeof(void*)));
  if (SYNC_MODE == COLLECTION_MODE_SYNCHRONIZED) pthread_mutex_init(&l->lock, nullptr);
  return l;
}

int array_list_clear(array_list_t* l, void (*data_callback)(void*)) {
  if (!l) return 0;
  if (data_callback)
    for (size_t i = 0; i < l->size; ++i)
      if (l->items[i]) data_callback(l->items[i]);
  l->size = 0;
  return 1;
}

void array_list_free(array_list_t* l, void (*data_callback)(void*)) {
  if (!l) return;
  array_list_clear(l, data_callback);
  if (l->mode == COLLECTION_MODE_SYNCHRONIZED) pthread_mutex_destroy(&l->lock);
  std::free(l->items);
  std::free(l);
}

int array_list_insert(void* item_p, array_list_t* l) {
  if (!l) return 0;
  lock(l);
  if (l->size >= l->capacity && !grow(l)) {
    unlock(l);
    return 0;
  }
  l->items[l->size++] = item_p;
  unlock(l);
  return 1;
}

size_t array_list_size(array_list_t* l) { return l ? l->size : 0; }

void* array_list_get(size_t index, array_list_t* l) {
  if (!l || index >= l->size) return nullptr;
  return l->items[index];
}

void* array_list_remove_at(size_t index, array_list_t* l) {
  if (!l || index >= l->size) return nullptr;
  lock(l);
  void* item = l->items[index];
  std::memmove(l->items + index, l->items + index + 1, (l->size - index - 1) * sizeof(void*));
  l->size--;
  unlock(l);
  return item;
}

void array_list_set_flag(int flag, array_list_t* l) {
  lock(l);
  l->flag = flag;
  unlock(l);
}

int array_list_get_flag(array_list_t* l) {
  lock(l);
  const int f = l->flag;
  unlock(l);
  return f;
}

alignment_t* alignment_new(void) { return static_cast<alignment_t*>(std::calloc(1, sizeof(alignment_t))); }

void alignment_free(alignment_t* a) {
  if (!a) return;
  std::free(a->query_name);
  std::free(a->sequence);
  std::free(a->quality);
  std::free(a->cigar);
  std::free(a->optional_fields);
  std::free(a);
}

linked_list_t* linked_list_new(int SYNC_MODE) {
  linked_list_t* l = static_cast<linked_list_t*>(std::calloc(1, sizeof(linked_list_t)));
  if (!l) return nullptr;
  l->mode = SYNC_MODE;
  if (SYNC_MODE == COLLECTION_MODE_SYNCHRONIZED) pthread_mutex_init(&l->lock, nullptr);
  return l;
}

void linked_list_free(linked_list_t* l, void (*data_callback)(void*)) {
  if (!l) return;
  for (linked_list_item_t* it = l->first; it;) {
    linked_list_item_t* next = it->next;
    if (data_callback && it->item) data_callback(it->item);
    std::free(it);
    it = next;
  }
  if (l->mode == COLLECTION_MODE_SYNCHRONIZED) pthread_mutex_destroy(&l->lock);
  std::free(l);
}

static linked_list_item_t* new_item(void* p) {
  linked_list_item_t* it = static_cast<linked_list_item_t*>(std::calloc(1, sizeof(linked_list_item_t)));
  if (it) it->item = p;
  return it;
}

int linked_list_insert(void* item_p, linked_list_t* l) {
  linked_list_item_t* it = new_item(item_p);
  if (!l || !it) return 0;
  if (l->mode == COLLECTION_MODE_SYNCHRONIZED) pthread_mutex_lock(&l->lock);
  it->next = l->first;
  if (l->first) l->first->prev = it;
  else l->last = it;
  l->first = it;
  l->size++;
  if (l->mode == COLLECTION_MODE_SYNCHRONIZED) pthread_mutex_unlock(&l->lock);
  return 1;
}

int linked_list_insert_last(void* item_p, linked_list_t* l) {
  linked_list_item_t* it = new_item(item_p);
  if (!l || !it) return 0;
  if (l->mode == COLLECTION_MODE_SYNCHRONIZED) pthread_mutex_lock(&l->lock);
  it->prev = l->last;
  if (l->last) l->last->next = it;
  else l->first = it;
  l->last = it;
  l->size++;
  if (l->mode == COLLECTION_MODE_SYNCHRONIZED) pthread_mutex_unlock(&l->lock);
  return 1;
}

size_t linked_list_size(linked_list_t* l) { return l ? l->size : 0; }

void* linked_list_get_first(linked_list_t* l) { return l && l->first ? l->first->item : nullptr; }

void* linked_list_get_last(linked_list_t* l) { return l && l->last ? l->last->item : nullptr; }

linked_list_iterator_t* linked_list_iterator_new(linked_list_t* l) {
  linked_list_iterator_t* it = static_cast<linked_list_iterator_t*>(std::malloc(sizeof(linked_list_iterator_t)));
  if (!it) return nullptr;
  it->linked_list_p = l;
  it->curr_pos = l ? l->first : nullptr;
  return it;
}

void linked_list_iterator_free(linked_list_iterator_t* it) { std::free(it); }

void* linked_list_iterator_curr(linked_list_iterator_t* it) { return it && it->curr_pos ? it->curr_pos->item : nullptr; }

void* linked_list_iterator_next(linked_list_iterator_t* it) {
  if (!it || !it->curr_pos) return nullptr;
  it->curr_pos = it->curr_pos->next;
  return it->curr_pos ? it->curr_pos->item : nullptr;
}

}  // extern "C"
